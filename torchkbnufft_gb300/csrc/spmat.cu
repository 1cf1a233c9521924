// Sparse-matrix interpolation: y = A x and x = A^H y with a caller-given
// complex interpolation matrix A (one row per k-space point, one column per
// grid cell), as torchkbnufft's spmat_interp / spmat_interp_adjoint
// (torchkbnufft/_nufft/interp.py:13-85) do with torch.mm on the matrix's real
// and imaginary parts. Forward: one thread per (plane, row) sums its row in
// CSR order. Adjoint: one thread per (plane, nonzero) adds its product into
// the grid with an atomic (the matrix may have any sparsity pattern).

#include "tkbn_common.cuh"

namespace tkbn {

template <typename R>
__global__ void k_spmat_fwd(int64_t nrows, int64_t ncols, int64_t nplanes, const int64_t* __restrict__ crow,
                            const int32_t* __restrict__ col, const cplx<R>* __restrict__ val,
                            const cplx<R>* __restrict__ x, cplx<R>* __restrict__ y) {
  const int64_t total = nrows * nplanes;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t plane = idx / nrows, row = idx - plane * nrows;
    const cplx<R>* xp = x + plane * ncols;
    cplx<R> acc = mk<R>(0, 0);
    for (int64_t e = crow[row]; e < crow[row + 1]; ++e) acc = cfma<R>(val[e], xp[col[e]], acc);
    y[idx] = acc;
  }
}

__device__ __forceinline__ void atomic_add_c(float2* p, float2 v) { atomicAdd(p, v); }
__device__ __forceinline__ void atomic_add_c(double2* p, double2 v) {
  atomicAdd(&p->x, v.x);
  atomicAdd(&p->y, v.y);
}

template <typename R>
__global__ void k_spmat_adj(int64_t nrows, int64_t ncols, int64_t nnz, int64_t nplanes,
                            const int32_t* __restrict__ row, const int32_t* __restrict__ col,
                            const cplx<R>* __restrict__ val, const cplx<R>* __restrict__ y, cplx<R>* __restrict__ x) {
  const int64_t total = nnz * nplanes;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t plane = idx / nnz, e = idx - plane * nnz;
    const cplx<R> v = cmulc<R>(y[plane * nrows + row[e]], val[e]);  // conj(a) * y
    atomic_add_c(x + plane * ncols + col[e], v);
  }
}

}  // namespace tkbn

namespace tkbn_host {

using namespace tkbn;

static int spmat_blocks(int64_t work) {
  int64_t b = (work + 255) / 256;
  if (b > 152 * 16) b = 152 * 16;
  return (int)(b < 1 ? 1 : b);
}

int spmat_interp(int dtype, int64_t nrows, int64_t ncols, const int64_t* crow, const int32_t* col, const void* val,
                 const void* x, int64_t nplanes, void* y, cudaStream_t s) {
  if (nrows < 0 || ncols < 1 || nplanes < 1) return set_error(TKBN_ERR_INVALID, "bad sparse matrix shape");
  if (nrows == 0) return TKBN_OK;
  if (!crow || !x || !y) return set_error(TKBN_ERR_INVALID, "null pointer argument");
  const int blocks = spmat_blocks(nrows * nplanes);
  if (dtype == TKBN_C64)
    k_spmat_fwd<float><<<blocks, 256, 0, s>>>(nrows, ncols, nplanes, crow, col, (const float2*)val, (const float2*)x,
                                              (float2*)y);
  else if (dtype == TKBN_C128)
    k_spmat_fwd<double><<<blocks, 256, 0, s>>>(nrows, ncols, nplanes, crow, col, (const double2*)val,
                                               (const double2*)x, (double2*)y);
  else
    return set_error(TKBN_ERR_UNSUPPORTED, "unsupported dtype %d", dtype);
  return check_cuda(cudaGetLastError(), "spmat interp launch");
}

int spmat_interp_adjoint(int dtype, int64_t nrows, int64_t ncols, int64_t nnz, const int32_t* row, const int32_t* col,
                         const void* val, const void* y, int64_t nplanes, void* x, cudaStream_t s) {
  if (nrows < 0 || ncols < 1 || nnz < 0 || nplanes < 1) return set_error(TKBN_ERR_INVALID, "bad sparse matrix shape");
  if (!x) return set_error(TKBN_ERR_INVALID, "null grid");
  const size_t esize = dtype == TKBN_C64 ? 8 : 16;
  int rc = check_cuda(cudaMemsetAsync(x, 0, (size_t)(ncols * nplanes) * esize, s), "zero grid");
  if (rc || nnz == 0) return rc;
  if (!row || !col || !val || !y) return set_error(TKBN_ERR_INVALID, "null pointer argument");
  const int blocks = spmat_blocks(nnz * nplanes);
  if (dtype == TKBN_C64)
    k_spmat_adj<float><<<blocks, 256, 0, s>>>(nrows, ncols, nnz, nplanes, row, col, (const float2*)val,
                                              (const float2*)y, (float2*)x);
  else if (dtype == TKBN_C128)
    k_spmat_adj<double><<<blocks, 256, 0, s>>>(nrows, ncols, nnz, nplanes, row, col, (const double2*)val,
                                               (const double2*)y, (double2*)x);
  else
    return set_error(TKBN_ERR_UNSUPPORTED, "unsupported dtype %d", dtype);
  return check_cuda(cudaGetLastError(), "spmat adjoint launch");
}

}  // namespace tkbn_host
