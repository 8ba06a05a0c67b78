// Output of a solution: VTU files for visual checks and a raw state file for
// restart, the part of the reference's output_results that writes
// "solution_NNN.vtu" through DataOut (advection_solver.cc:1220-1241).
//
// VTU: an UnstructuredGrid with the (k+1)^3 Gauss-Lobatto support points of
// every cell (mapped, so curved cells are resolved at the nodes; points are
// not shared between cells because the field is discontinuous), each cell
// split into k^3 trilinear hexahedra over its nodes (DataOut with fe_degree
// subdivisions; the reference writes the same nodes as one Lagrange cell),
// and the point fields "solution" (the nodal values, which are the DoFs) and
// "analytic_solution" (the exact solution at the nodes at the given time).
//
// Raw state: a 64-byte header (magic "ADVSTAT1", degree, cells per
// direction, mesh type, time, number of values) followed by the owned nodal
// values in the library's layout; adv_load_state checks the header against
// the handle.
#include <cstdio>
#include <cstring>
#include <vector>

#include "geometry.h"
#include "handle.h"
#include "kernels.h"
#include "tables.h"

using adv::detail::fail;

namespace
{
struct StateHeader
{
  char    magic[8];
  int32_t degree, n_cells[3], mesh_type, reserved;
  double  time;
  int64_t n_values;
  int64_t pad[2];
};
static_assert(sizeof(StateHeader) == 64, "state header is 64 bytes");

// values of the owned cells: local cells [cell_begin, cell_end) of the mesh m
int write_vtu(const adv_config &cfg, const adv::Mesh &m, const double *vals, double time, const char *path)
{
  FILE *f = std::fopen(path, "w");
  if (!f)
    return fail(ADV_ERR_INVALID, "cannot open the output file");
  adv::Tables1D tb;
  tb.init(cfg.degree);
  adv::DiagArgs g;
  adv::detail::make_diag(cfg, m, tb, g);
  const int     n = m.n, nq = n * n * n, k = n - 1;
  const int64_t cells = m.cell_end - m.cell_begin;
  const int64_t npts = cells * nq, nhex = cells * (int64_t)k * k * k;
  std::fprintf(f, "<?xml version=\"1.0\"?>\n<VTKFile type=\"UnstructuredGrid\" version=\"0.1\" "
                  "byte_order=\"LittleEndian\">\n<UnstructuredGrid>\n");
  std::fprintf(f, "<FieldData><DataArray type=\"Float64\" Name=\"TIME\" NumberOfTuples=\"1\" "
                  "format=\"ascii\">%.17g</DataArray></FieldData>\n", time);
  std::fprintf(f, "<Piece NumberOfPoints=\"%lld\" NumberOfCells=\"%lld\">\n", (long long)npts, (long long)nhex);
  std::vector<double> X(3 * nq);
  std::fprintf(f, "<Points><DataArray type=\"Float64\" NumberOfComponents=\"3\" format=\"ascii\">\n");
  for (int64_t c = m.cell_begin; c < m.cell_end; ++c)
    {
      adv::support_points(cfg, m, tb, c, X.data());
      for (int i = 0; i < nq; ++i)
        std::fprintf(f, "%.17g %.17g %.17g\n", X[3 * i], X[3 * i + 1], X[3 * i + 2]);
    }
  std::fprintf(f, "</DataArray></Points>\n<Cells>\n<DataArray type=\"Int64\" Name=\"connectivity\" "
                  "format=\"ascii\">\n");
  for (int64_t c = 0; c < cells; ++c)
    for (int kz = 0; kz < k; ++kz)
      for (int ky = 0; ky < k; ++ky)
        for (int kx = 0; kx < k; ++kx)
          {
            const int64_t b = c * nq;
            auto          p = [&](int a, int bb, int cc) { return b + a + n * (bb + n * cc); };
            std::fprintf(f, "%lld %lld %lld %lld %lld %lld %lld %lld\n", (long long)p(kx, ky, kz),
                         (long long)p(kx + 1, ky, kz), (long long)p(kx + 1, ky + 1, kz), (long long)p(kx, ky + 1, kz),
                         (long long)p(kx, ky, kz + 1), (long long)p(kx + 1, ky, kz + 1),
                         (long long)p(kx + 1, ky + 1, kz + 1), (long long)p(kx, ky + 1, kz + 1));
          }
  std::fprintf(f, "</DataArray>\n<DataArray type=\"Int64\" Name=\"offsets\" format=\"ascii\">\n");
  for (int64_t h = 1; h <= nhex; ++h)
    std::fprintf(f, "%lld\n", (long long)(8 * h));
  std::fprintf(f, "</DataArray>\n<DataArray type=\"UInt8\" Name=\"types\" format=\"ascii\">\n");
  for (int64_t h = 0; h < nhex; ++h)
    std::fprintf(f, "12\n");
  std::fprintf(f, "</DataArray>\n</Cells>\n<PointData Scalars=\"solution\">\n"
                  "<DataArray type=\"Float64\" Name=\"solution\" format=\"ascii\">\n");
  for (int64_t i = 0; i < npts; ++i)
    std::fprintf(f, "%.17g\n", vals[i]);
  std::fprintf(f, "</DataArray>\n<DataArray type=\"Float64\" Name=\"analytic_solution\" format=\"ascii\">\n");
  for (int64_t c = m.cell_begin; c < m.cell_end; ++c)
    {
      adv::support_points(cfg, m, tb, c, X.data());
      for (int i = 0; i < nq; ++i)
        std::fprintf(f, "%.17g\n", adv::exact_value(g.ex, X[3 * i], X[3 * i + 1], X[3 * i + 2], time));
    }
  std::fprintf(f, "</DataArray>\n</PointData>\n</Piece>\n</UnstructuredGrid>\n</VTKFile>\n");
  const bool ok = std::ferror(f) == 0;
  std::fclose(f);
  return ok ? ADV_OK : fail(ADV_ERR_INVALID, "write error on the output file");
}

int copy_owned(adv_handle *h, const double *dev, std::vector<double> &host, void *stream)
{
  const int64_t n3 = (int64_t)h->mesh.n * h->mesh.n * h->mesh.n;
  host.resize((h->mesh.cell_end - h->mesh.cell_begin) * n3);
  ADV_CUDA(cudaMemcpyAsync(host.data(), dev + h->mesh.cell_begin * n3, host.size() * sizeof(double),
                           cudaMemcpyDeviceToHost, (cudaStream_t)stream));
  ADV_CUDA(cudaStreamSynchronize((cudaStream_t)stream));
  return ADV_OK;
}
} // namespace

extern "C" {

int adv_write_vtu(adv_handle *h, const double *vec, double time, const char *path, void *stream)
{
  if (!h || !vec || !path)
    return fail(ADV_ERR_INVALID, "null argument");
  std::vector<double> host;
  if (int e = copy_owned(h, vec, host, stream))
    return e;
  return write_vtu(h->cfg, h->mesh, host.data(), time, path);
}

int adv_write_vtu_host(const adv_config *cfg, const double *host_vec, double time, const char *path)
{
  if (!cfg || !host_vec || !path)
    return fail(ADV_ERR_INVALID, "null argument");
  if (cfg->degree < 1 || cfg->degree > 6 || cfg->n_cells[0] < 1 || cfg->n_cells[1] < 1 || cfg->n_cells[2] < 1)
    return fail(ADV_ERR_INVALID, "bad configuration");
  adv::Mesh m;
  adv::setup_mesh(*cfg, m);
  return write_vtu(*cfg, m, host_vec, time, path);
}

int adv_save_state(adv_handle *h, const double *vec, double time, const char *path, void *stream)
{
  if (!h || !vec || !path)
    return fail(ADV_ERR_INVALID, "null argument");
  std::vector<double> host;
  if (int e = copy_owned(h, vec, host, stream))
    return e;
  StateHeader hd;
  std::memset(&hd, 0, sizeof(hd));
  std::memcpy(hd.magic, "ADVSTAT1", 8);
  hd.degree = h->cfg.degree;
  for (int d = 0; d < 3; ++d)
    hd.n_cells[d] = h->cfg.n_cells[d];
  hd.mesh_type = h->cfg.mesh_type;
  hd.time      = time;
  hd.n_values  = (int64_t)host.size();
  FILE *f      = std::fopen(path, "wb");
  if (!f)
    return fail(ADV_ERR_INVALID, "cannot open the state file");
  const bool ok = std::fwrite(&hd, sizeof(hd), 1, f) == 1 &&
                  std::fwrite(host.data(), sizeof(double), host.size(), f) == host.size();
  std::fclose(f);
  return ok ? ADV_OK : fail(ADV_ERR_INVALID, "write error on the state file");
}

int adv_load_state(adv_handle *h, double *vec, double *time, const char *path, void *stream)
{
  if (!h || !vec || !path)
    return fail(ADV_ERR_INVALID, "null argument");
  FILE *f = std::fopen(path, "rb");
  if (!f)
    return fail(ADV_ERR_INVALID, "cannot open the state file");
  StateHeader hd;
  const int64_t n3    = (int64_t)h->mesh.n * h->mesh.n * h->mesh.n;
  const int64_t owned = (h->mesh.cell_end - h->mesh.cell_begin) * n3;
  bool ok = std::fread(&hd, sizeof(hd), 1, f) == 1 && std::memcmp(hd.magic, "ADVSTAT1", 8) == 0;
  ok      = ok && hd.degree == h->cfg.degree && hd.mesh_type == h->cfg.mesh_type && hd.n_values == owned;
  for (int d = 0; d < 3; ++d)
    ok = ok && hd.n_cells[d] == h->cfg.n_cells[d];
  std::vector<double> host;
  if (ok)
    {
      host.resize(owned);
      ok = std::fread(host.data(), sizeof(double), owned, f) == (size_t)owned;
    }
  std::fclose(f);
  if (!ok)
    return fail(ADV_ERR_INVALID, "state file does not match this operator (degree, mesh, size) or is truncated");
  ADV_CUDA(cudaMemcpyAsync(vec + h->mesh.cell_begin * n3, host.data(), owned * sizeof(double),
                           cudaMemcpyHostToDevice, (cudaStream_t)stream));
  ADV_CUDA(cudaStreamSynchronize((cudaStream_t)stream));
  if (time)
    *time = hd.time;
  return ADV_OK;
}

} // extern "C"
