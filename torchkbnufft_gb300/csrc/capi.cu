// extern "C" entry points of include/tkbn_gb300.h: argument checks and
// dispatch to the implementation units. No allocation happens here.

#include <exception>

#include "tkbn_common.cuh"

namespace tkbn_host {
const char* last_error();
int points_build(const tkbn_geometry* g, const tkbn_points_desc* p, const void* omega, void* ws, size_t bytes,
                 cudaStream_t s);
int interp_fwd(const tkbn_geometry* g, const tkbn_points_desc* p, const void* ws, const void* const* tables,
               const void* grid, int64_t B, int64_t C, void* kdata, cudaStream_t s);
int interp_adj(const tkbn_geometry* g, const tkbn_points_desc* p, const void* ws, const void* const* tables,
               const void* kdata, int64_t B, int64_t C, void* grid, cudaStream_t s);
int interp_grad(const tkbn_geometry* g, const tkbn_points_desc* p, const void* ws, const void* const* tables,
                const void* const* dtables, const void* grid, const void* v, int64_t B, int64_t C, void* grad,
                cudaStream_t s);
int fft_plan_create(const tkbn_geometry* g, int64_t B, int64_t C, tkbn_fft_plan* out);
int fft_plan_destroy(tkbn_fft_plan p);
int fft_and_scale(const tkbn_geometry* g, tkbn_fft_plan plan, const void* image, const void* smaps,
                  int64_t smaps_batch, const void* scaling, int64_t B, int64_t C, int norm, void* grid,
                  cudaStream_t st);
int ifft_and_scale(const tkbn_geometry* g, tkbn_fft_plan plan, void* grid, const void* smaps, int64_t smaps_batch,
                   const void* scaling, int64_t B, int64_t C, int norm, void* image, cudaStream_t st);
int toep_apply(const tkbn_geometry* g, tkbn_fft_plan plan, const void* image, const void* kernel, int64_t kbatch,
               int by_channel, const void* smaps, int64_t smaps_batch, int64_t B, int64_t C, int norm, void* grid,
               void* out, cudaStream_t st);
int spmat_interp(int dtype, int64_t nrows, int64_t ncols, const int64_t* crow, const int32_t* col, const void* val,
                 const void* x, int64_t nplanes, void* y, cudaStream_t s);
int spmat_interp_adjoint(int dtype, int64_t nrows, int64_t ncols, int64_t nnz, const int32_t* row, const int32_t* col,
                         const void* val, const void* y, int64_t nplanes, void* x, cudaStream_t s);
int toep_assemble(int dtype, int ndim, const int64_t* im_size, const void* parts, double scale, void* out,
                  cudaStream_t s);
int ragged_plan_create(const tkbn_ragged_problem* pr, int64_t n, tkbn_ragged_plan* out);
int ragged_plan_destroy(tkbn_ragged_plan p);
int ragged_interp_fwd(tkbn_ragged_plan p, cudaStream_t s);
int ragged_interp_adj(tkbn_ragged_plan p, cudaStream_t s);
}  // namespace tkbn_host

using namespace tkbn_host;

#define TKBN_GUARD(expr)                                                  \
  try {                                                                   \
    return (expr);                                                        \
  } catch (const std::exception& e) {                                     \
    return set_error(TKBN_ERR_INVALID, "internal error: %s", e.what());   \
  } catch (...) {                                                         \
    return set_error(TKBN_ERR_INVALID, "internal error");                 \
  }

static int check_geometry(const tkbn_geometry* g) {
  if (!g) return set_error(TKBN_ERR_INVALID, "geometry is null");
  if (g->ndim < 1 || g->ndim > 3) return set_error(TKBN_ERR_UNSUPPORTED, "ndim must be 1, 2 or 3 (got %d)", g->ndim);
  if (g->dtype != TKBN_C64 && g->dtype != TKBN_C128)
    return set_error(TKBN_ERR_UNSUPPORTED, "dtype must be complex64 or complex128");
  for (int d = 0; d < g->ndim; ++d) {
    if (g->grid_size[d] < 1 || g->grid_size[d] > (1 << 24)) return set_error(TKBN_ERR_INVALID, "bad grid_size");
    if (g->im_size[d] < 1) return set_error(TKBN_ERR_INVALID, "bad im_size");
  }
  return TKBN_OK;
}

static int check_tables(const tkbn_geometry* g, const void* const* t) {
  if (!t) return set_error(TKBN_ERR_INVALID, "tables is null");
  for (int d = 0; d < g->ndim; ++d)
    if (!t[d]) return set_error(TKBN_ERR_INVALID, "table %d is null", d);
  return TKBN_OK;
}

extern "C" {

int tkbn_abi_version(void) { return TKBN_ABI_VERSION; }

const char* tkbn_last_error(void) { return last_error(); }

int tkbn_device_status(void* stream, int32_t* status) {
  if (!status) return set_error(TKBN_ERR_INVALID, "status is null");
  int st = 0, rc;
  cudaStream_t s = (cudaStream_t)stream;
  if ((rc = status_points(s, &st)) || (rc = status_interp(s, &st)) || (rc = status_fft(s, &st))) return rc;
  *status = st;
  return TKBN_OK;
}

int tkbn_points_workspace_size(const tkbn_geometry* g, const tkbn_points_desc* p, size_t* bytes) {
  int rc = check_geometry(g);
  if (rc) return rc;
  if (!bytes) return set_error(TKBN_ERR_INVALID, "bytes is null");
  PointsLayout L;
  TKBN_GUARD((rc = points_layout(g, p, &L), rc == TKBN_OK ? (*bytes = L.total, TKBN_OK) : rc));
}

int tkbn_points_build(const tkbn_geometry* g, const tkbn_points_desc* p, const void* omega, void* workspace,
                      size_t workspace_bytes, void* stream) {
  int rc = check_geometry(g);
  if (rc) return rc;
  TKBN_GUARD(points_build(g, p, omega, workspace, workspace_bytes, (cudaStream_t)stream));
}

int tkbn_interp_fwd(const tkbn_geometry* g, const tkbn_points_desc* p, const void* workspace,
                    const void* const* tables, const void* grid, int64_t nbatch, int64_t ncoil, void* kdata,
                    void* stream) {
  int rc = check_geometry(g);
  if (rc || (rc = check_tables(g, tables))) return rc;
  if (!p) return set_error(TKBN_ERR_INVALID, "points desc is null");
  if (p->npts > 0 && (!grid || !kdata)) return set_error(TKBN_ERR_INVALID, "null grid or kdata");
  TKBN_GUARD(interp_fwd(g, p, workspace, tables, grid, nbatch, ncoil, kdata, (cudaStream_t)stream));
}

int tkbn_interp_adj(const tkbn_geometry* g, const tkbn_points_desc* p, const void* workspace,
                    const void* const* tables, const void* kdata, int64_t nbatch, int64_t ncoil, void* grid,
                    void* stream) {
  int rc = check_geometry(g);
  if (rc || (rc = check_tables(g, tables))) return rc;
  if (!p) return set_error(TKBN_ERR_INVALID, "points desc is null");
  if (!grid || (p->npts > 0 && !kdata)) return set_error(TKBN_ERR_INVALID, "null grid or kdata");
  TKBN_GUARD(interp_adj(g, p, workspace, tables, kdata, nbatch, ncoil, grid, (cudaStream_t)stream));
}

int tkbn_interp_grad_omega(const tkbn_geometry* g, const tkbn_points_desc* p, const void* workspace,
                           const void* const* tables, const void* const* dtables, const void* grid, const void* v,
                           int64_t nbatch, int64_t ncoil, void* grad_omega, void* stream) {
  int rc = check_geometry(g);
  if (rc || (rc = check_tables(g, tables)) || (rc = check_tables(g, dtables))) return rc;
  if (!p) return set_error(TKBN_ERR_INVALID, "points desc is null");
  if (!grad_omega || (p->npts > 0 && (!grid || !v))) return set_error(TKBN_ERR_INVALID, "null pointer argument");
  TKBN_GUARD(interp_grad(g, p, workspace, tables, dtables, grid, v, nbatch, ncoil, grad_omega, (cudaStream_t)stream));
}

int tkbn_fft_plan_create(const tkbn_geometry* g, int64_t nbatch, int64_t ncoil, tkbn_fft_plan* plan) {
  int rc = check_geometry(g);
  if (rc) return rc;
  TKBN_GUARD(fft_plan_create(g, nbatch, ncoil, plan));
}

int tkbn_fft_plan_destroy(tkbn_fft_plan plan) { TKBN_GUARD(fft_plan_destroy(plan)); }

int tkbn_fft_and_scale(const tkbn_geometry* g, tkbn_fft_plan plan, const void* image, const void* smaps,
                       int64_t smaps_batch, const void* scaling, int64_t nbatch, int64_t ncoil, int norm, void* grid,
                       void* stream) {
  int rc = check_geometry(g);
  if (rc) return rc;
  TKBN_GUARD(fft_and_scale(g, plan, image, smaps, smaps_batch, scaling, nbatch, ncoil, norm, grid, (cudaStream_t)stream));
}

int tkbn_ifft_and_scale(const tkbn_geometry* g, tkbn_fft_plan plan, void* grid, const void* smaps,
                        int64_t smaps_batch, const void* scaling, int64_t nbatch, int64_t ncoil, int norm, void* image,
                        void* stream) {
  int rc = check_geometry(g);
  if (rc) return rc;
  TKBN_GUARD(ifft_and_scale(g, plan, grid, smaps, smaps_batch, scaling, nbatch, ncoil, norm, image, (cudaStream_t)stream));
}

int tkbn_nufft_fwd(const tkbn_geometry* g, const tkbn_points_desc* p, const void* workspace, tkbn_fft_plan plan,
                   const void* const* tables, const void* scaling, const void* image, const void* smaps,
                   int64_t smaps_batch, int64_t nbatch, int64_t ncoil, int norm, void* grid_scratch, void* kdata,
                   void* stream) {
  int rc = tkbn_fft_and_scale(g, plan, image, smaps, smaps_batch, scaling, nbatch, ncoil, norm, grid_scratch, stream);
  if (rc) return rc;
  return tkbn_interp_fwd(g, p, workspace, tables, grid_scratch, nbatch, ncoil, kdata, stream);
}

int tkbn_nufft_adj(const tkbn_geometry* g, const tkbn_points_desc* p, const void* workspace, tkbn_fft_plan plan,
                   const void* const* tables, const void* scaling, const void* kdata, const void* smaps,
                   int64_t smaps_batch, int64_t nbatch, int64_t ncoil, int norm, void* grid_scratch, void* image,
                   void* stream) {
  int rc = tkbn_interp_adj(g, p, workspace, tables, kdata, nbatch, ncoil, grid_scratch, stream);
  if (rc) return rc;
  return tkbn_ifft_and_scale(g, plan, grid_scratch, smaps, smaps_batch, scaling, nbatch, ncoil, norm, image, stream);
}

int tkbn_fft_filter(const tkbn_geometry* g, tkbn_fft_plan plan, const void* image, const void* kernel,
                    int64_t kernel_batch, int64_t nbatch, int64_t ncoil, int norm, void* grid_scratch, void* out,
                    void* stream) {
  int rc = check_geometry(g);
  if (rc) return rc;
  TKBN_GUARD(toep_apply(g, plan, image, kernel, kernel_batch, 1, nullptr, 1, nbatch, ncoil, norm, grid_scratch, out,
                        (cudaStream_t)stream));
}

int tkbn_toep_apply(const tkbn_geometry* g, tkbn_fft_plan plan, const void* image, const void* kernel,
                    int64_t kernel_batch, const void* smaps, int64_t smaps_batch, int64_t nbatch, int64_t ncoil,
                    int norm, void* grid_scratch, void* out, void* stream) {
  int rc = check_geometry(g);
  if (rc) return rc;
  if (!smaps) return set_error(TKBN_ERR_INVALID, "smaps is null (use tkbn_fft_filter without maps)");
  TKBN_GUARD(toep_apply(g, plan, image, kernel, kernel_batch, 0, smaps, smaps_batch, nbatch, ncoil, norm,
                        grid_scratch, out, (cudaStream_t)stream));
}

int tkbn_toep_kernel_assemble(int dtype, int ndim, const int64_t* im_size, const void* parts, double scale,
                              void* out, void* stream) {
  if (parts && out && parts == out) return set_error(TKBN_ERR_INVALID, "out must not alias parts");
  TKBN_GUARD(toep_assemble(dtype, ndim, im_size, parts, scale, out, (cudaStream_t)stream));
}

}  // extern "C"

int tkbn_ragged_plan_create(const tkbn_ragged_problem* problems, int64_t nproblems, tkbn_ragged_plan* plan) {
  if (!problems || !plan) return set_error(TKBN_ERR_INVALID, "null argument");
  TKBN_GUARD(ragged_plan_create(problems, nproblems, plan));
}

int tkbn_ragged_plan_destroy(tkbn_ragged_plan plan) { TKBN_GUARD(ragged_plan_destroy(plan)); }

int tkbn_ragged_interp_fwd(tkbn_ragged_plan plan, void* stream) {
  TKBN_GUARD(ragged_interp_fwd(plan, (cudaStream_t)stream));
}

int tkbn_ragged_interp_adj(tkbn_ragged_plan plan, void* stream) {
  TKBN_GUARD(ragged_interp_adj(plan, (cudaStream_t)stream));
}

int tkbn_spmat_interp(int dtype, int64_t nrows, int64_t ncols, const int64_t* crow, const int32_t* col,
                      const void* val, const void* x, int64_t nplanes, void* y, void* stream) {
  TKBN_GUARD(spmat_interp(dtype, nrows, ncols, crow, col, val, x, nplanes, y, (cudaStream_t)stream));
}

int tkbn_spmat_interp_adjoint(int dtype, int64_t nrows, int64_t ncols, int64_t nnz, const int32_t* row,
                              const int32_t* col, const void* val, const void* y, int64_t nplanes, void* x,
                              void* stream) {
  TKBN_GUARD(spmat_interp_adjoint(dtype, nrows, ncols, nnz, row, col, val, y, nplanes, x, (cudaStream_t)stream));
}
