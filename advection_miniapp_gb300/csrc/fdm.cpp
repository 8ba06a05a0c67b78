#include "fdm.h"

#include <algorithm>
#include <cmath>

#include "tables.h"

namespace adv
{
namespace
{
using cd = std::complex<double>;

// reduction to upper Hessenberg form by Householder reflections (in place, row-major)
void hessenberg(int n, std::vector<cd> &H)
{
  for (int k = 0; k < n - 2; ++k)
    {
      double norm2 = 0.0;
      for (int i = k + 1; i < n; ++i)
        norm2 += std::norm(H[i * n + k]);
      const double alpha = std::sqrt(norm2);
      if (alpha == 0.0)
        continue;
      const cd        x0    = H[(k + 1) * n + k];
      const cd        phase = std::abs(x0) == 0.0 ? cd(1.0) : x0 / std::abs(x0);
      std::vector<cd> v(n - k - 1);
      for (int i = 0; i < n - k - 1; ++i)
        v[i] = H[(k + 1 + i) * n + k];
      v[0] += phase * alpha;
      double vn = 0.0;
      for (auto &x : v)
        vn += std::norm(x);
      if (vn == 0.0)
        continue;
      for (int j = 0; j < n; ++j)
        {
          cd s = 0.0;
          for (int i = 0; i < n - k - 1; ++i)
            s += std::conj(v[i]) * H[(k + 1 + i) * n + j];
          s *= 2.0 / vn;
          for (int i = 0; i < n - k - 1; ++i)
            H[(k + 1 + i) * n + j] -= v[i] * s;
        }
      for (int i = 0; i < n; ++i)
        {
          cd s = 0.0;
          for (int j = 0; j < n - k - 1; ++j)
            s += H[i * n + k + 1 + j] * v[j];
          s *= 2.0 / vn;
          for (int j = 0; j < n - k - 1; ++j)
            H[i * n + k + 1 + j] -= s * std::conj(v[j]);
        }
    }
}

// eigenvalues of an upper Hessenberg matrix by shifted QR with Givens rotations
bool hessenberg_qr(int n, std::vector<cd> &H, std::vector<cd> &lambda)
{
  const double eps  = 1e-15;
  int          hi   = n - 1;
  int          iter = 0;
  while (hi > 0)
    {
      int l = hi;
      while (l > 0 && std::abs(H[l * n + l - 1]) > eps * (std::abs(H[l * n + l]) + std::abs(H[(l - 1) * n + l - 1])))
        --l;
      if (l == hi)
        {
          --hi;
          iter = 0;
          continue;
        }
      if (++iter > 500)
        return false;
      // Wilkinson shift from the trailing 2 x 2 block
      const cd a = H[(hi - 1) * n + hi - 1], b = H[(hi - 1) * n + hi], c = H[hi * n + hi - 1], d = H[hi * n + hi];
      const cd tr = a + d, det = a * d - b * c;
      const cd disc = std::sqrt(tr * tr / 4.0 - det);
      const cd mu1 = tr / 2.0 + disc, mu2 = tr / 2.0 - disc;
      cd       mu  = std::abs(mu1 - d) < std::abs(mu2 - d) ? mu1 : mu2;
      if (iter % 11 == 10)
        mu += std::abs(H[hi * n + hi - 1]); // exceptional shift
      for (int k = l; k <= hi; ++k)
        H[k * n + k] -= mu;
      std::vector<cd> cs(hi - l), sn(hi - l);
      for (int k = l; k < hi; ++k)
        {
          const cd     x = H[k * n + k], y = H[(k + 1) * n + k];
          const double r = std::sqrt(std::norm(x) + std::norm(y));
          cd           cc, ss;
          if (r == 0.0)
            cc = 1.0, ss = 0.0;
          else if (std::abs(x) == 0.0)
            cc = 0.0, ss = 1.0;
          else
            {
              cc = std::abs(x) / r;
              ss = (x / std::abs(x)) * std::conj(y) / r;
            }
          cs[k - l] = cc, sn[k - l] = ss;
          // rows k, k+1:  [c s; -conj(s) c]
          for (int j = k; j < n; ++j)
            {
              const cd p = H[k * n + j], q = H[(k + 1) * n + j];
              H[k * n + j]       = cc * p + ss * q;
              H[(k + 1) * n + j] = -std::conj(ss) * p + cc * q;
            }
        }
      for (int k = l; k < hi; ++k)
        {
          const cd cc = cs[k - l], ss = sn[k - l];
          // columns k, k+1 with the conjugate transpose of the rotation
          for (int i = 0; i <= std::min(k + 2, hi); ++i)
            {
              const cd p = H[i * n + k], q = H[i * n + k + 1];
              H[i * n + k]     = p * std::conj(cc) + q * std::conj(ss);
              H[i * n + k + 1] = -p * ss + q * std::conj(cc);
            }
        }
      for (int k = l; k <= hi; ++k)
        H[k * n + k] += mu;
    }
  lambda.resize(n);
  for (int i = 0; i < n; ++i)
    lambda[i] = H[i * n + i];
  return true;
}

// solve M x = b (complex, partial pivoting); M is destroyed
bool solve(int n, std::vector<cd> M, std::vector<cd> &x)
{
  for (int c = 0; c < n; ++c)
    {
      int p = c;
      for (int r = c + 1; r < n; ++r)
        if (std::abs(M[r * n + c]) > std::abs(M[p * n + c]))
          p = r;
      if (std::abs(M[p * n + c]) == 0.0)
        return false;
      if (p != c)
        {
          for (int j = 0; j < n; ++j)
            std::swap(M[c * n + j], M[p * n + j]);
          std::swap(x[c], x[p]);
        }
      for (int r = c + 1; r < n; ++r)
        {
          const cd f = M[r * n + c] / M[c * n + c];
          for (int j = c; j < n; ++j)
            M[r * n + j] -= f * M[c * n + j];
          x[r] -= f * x[c];
        }
    }
  for (int r = n - 1; r >= 0; --r)
    {
      cd s = x[r];
      for (int j = r + 1; j < n; ++j)
        s -= M[r * n + j] * x[j];
      x[r] = s / M[r * n + r];
    }
  return true;
}

bool invert(int n, const std::vector<cd> &A, std::vector<cd> &inv)
{
  inv.assign(n * n, 0.0);
  for (int j = 0; j < n; ++j)
    {
      std::vector<cd> e(n, 0.0);
      e[j] = 1.0;
      if (!solve(n, A, e))
        return false;
      for (int i = 0; i < n; ++i)
        inv[i * n + j] = e[i];
    }
  return true;
}
} // namespace

bool eigen_small(int n, const std::vector<cd> &A, std::vector<cd> &lambda, std::vector<cd> &V)
{
  std::vector<cd> H = A;
  hessenberg(n, H);
  if (!hessenberg_qr(n, H, lambda))
    return false;
  double anorm = 0.0;
  for (const auto &a : A)
    anorm = std::max(anorm, std::abs(a));
  V.assign(n * n, 0.0);
  for (int k = 0; k < n; ++k)
    {
      // inverse iteration with a slightly perturbed eigenvalue
      const cd        mu = lambda[k] + cd(1e-10, 1e-10) * std::max(1.0, anorm);
      std::vector<cd> M(A), x(n);
      for (int i = 0; i < n; ++i)
        {
          M[i * n + i] -= mu;
          x[i] = cd(1.0 + 0.1 * i, 0.05 * i);
        }
      for (int it = 0; it < 4; ++it)
        {
          if (!solve(n, M, x))
            return false;
          double nrm = 0.0;
          for (auto &v : x)
            nrm += std::norm(v);
          nrm = std::sqrt(nrm);
          for (auto &v : x)
            v /= nrm;
        }
      for (int i = 0; i < n; ++i)
        V[i * n + k] = x[i];
    }
  return true;
}

bool fdm_tables(int degree, double flux_alpha, FdmTables &t)
{
  Tables1D tb;
  tb.init(degree);
  const int n = tb.n;
  t.n         = n;
  t.residual  = 0.0;
  for (int si = 0; si < 2; ++si)
    {
      const double    s = si == 0 ? 1.0 : -1.0;
      std::vector<cd> A(n * n);
      t.A1[si].assign(n * n, 0.0);
      for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j)
          {
            // test function l_i, trial l_j; l_i'(g_j) = D[j][i], l_j(g_q) = delta_jq
            double a = -tb.D[j][i] * tb.gw[j] - tb.l0[i] * tb.l0[j] * 0.5 * (1.0 - flux_alpha * s) +
                       tb.l1[i] * tb.l1[j] * 0.5 * (1.0 + flux_alpha * s);
            a /= tb.gw[i];
            t.A1[si][i * n + j] = a;
            A[i * n + j]        = a;
          }
      std::vector<cd> lam, V, Vinv;
      if (!eigen_small(n, A, lam, V) || !invert(n, V, Vinv))
        return false;
      double anorm = 0.0, res = 0.0;
      for (int i = 0; i < n; ++i)
        for (int k = 0; k < n; ++k)
          {
            cd s2 = 0.0;
            for (int j = 0; j < n; ++j)
              s2 += A[i * n + j] * V[j * n + k];
            res   = std::max(res, std::abs(s2 - V[i * n + k] * lam[k]));
            anorm = std::max(anorm, std::abs(A[i * n + k]));
          }
      t.residual     = std::max(t.residual, res / anorm);
      t.lambda[si]   = lam;
      t.V[si]        = V;
      t.VinvW[si].assign(n * n, 0.0);
      for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j)
          t.VinvW[si][i * n + j] = Vinv[i * n + j] / tb.gw[j];
    }
  return t.residual < 1e-9;
}
} // namespace adv
