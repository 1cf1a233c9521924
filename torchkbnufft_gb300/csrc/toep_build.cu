// Toeplitz kernel assembly (calc_toeplitz_kernel, torchkbnufft/_nufft/toep.py:
// 11-307): from the 2^(d-1) sign-flipped adjoint NUFFTs of the weights, the
// Hermitian, scaled kernel on the (2N)^d grid in one pass, before its FFT.
//
// The reference builds it in steps: adjoint_flip_and_concat (toep.py:185-237)
// concatenates, along every image dim but the first, the part of the current
// flip pattern, a zero plane and the mirrored part of the pattern with that
// dim flipped; reflect_conj_concat (toep.py:240-274) appends along the first
// dim a zero plane and the conjugate point reflection; hermitify
// (toep.py:277-307) averages with the conjugate point reflection. Written
// per output cell u of the (2N)^d grid, with neg(u)_d = (2 N_d - u_d) mod 2 N_d:
//
//   A(u)  (u_0 < N_0): zero if u_d == N_d for some d >= 1; else part p at
//         (u_0, i_1, .., i_{d-1}) with i_d = u_d, bit d of p clear when
//         u_d < N_d, and i_d = 2 N_d - u_d, bit d set when u_d > N_d
//   K(u)  = A(u) for u_0 < N_0, 0 for u_0 == N_0, conj(A(2 N_0 - u_0, neg(u)_1, ..))
//   out(u) = scale * (K(u) + conj(K(neg(u)))) / 2
//
// so each output cell reads at most two part values and is written once.
// Part p of the pattern with dims 1..d-1 flipped according to bits
// (b_1 .. b_{d-1}) sits at index sum_d b_d 2^(d-1-d'), the order of the
// reference recursion (itertools.product over the flip bits).

#include "tkbn_common.cuh"

namespace tkbn {

struct ToepAsm {
  int nd;
  int N[3];
  int64_t pstride;  // elements per part (prod N)
};

// K(u): the reflected, flip-concatenated kernel before symmetrisation.
template <typename R>
__device__ __forceinline__ cplx<R> toep_K(const ToepAsm& a, const cplx<R>* __restrict__ parts, const int* u) {
  int v[3] = {u[0], u[1], u[2]};
  bool conj = false;
  if (v[0] == a.N[0]) return mk<R>(0, 0);
  if (v[0] > a.N[0]) {
    conj = true;
    v[0] = 2 * a.N[0] - v[0];
    for (int d = 1; d < a.nd; ++d) v[d] = v[d] == 0 ? 0 : 2 * a.N[d] - v[d];
  }
  int p = 0;
  int64_t off = v[0];
  for (int d = 1; d < a.nd; ++d) {
    int i = v[d];
    p <<= 1;
    if (i == a.N[d]) return mk<R>(0, 0);
    if (i > a.N[d]) {
      i = 2 * a.N[d] - i;
      p |= 1;
    }
    off = off * a.N[d] + i;
  }
  const cplx<R> z = parts[(int64_t)p * a.pstride + off];
  return conj ? mk<R>(z.x, -z.y) : z;
}

template <typename R>
__global__ void k_toep_assemble(ToepAsm a, const cplx<R>* __restrict__ parts, R scale, cplx<R>* __restrict__ out) {
  int64_t total = 1;
  for (int d = 0; d < a.nd; ++d) total *= 2 * a.N[d];
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < total; q += (int64_t)gridDim.x * blockDim.x) {
    int u[3] = {0, 0, 0}, w[3] = {0, 0, 0};
    int64_t r = q;
    for (int d = a.nd - 1; d >= 0; --d) {
      const int G = 2 * a.N[d];
      u[d] = (int)(r % G);
      r /= G;
      w[d] = u[d] == 0 ? 0 : G - u[d];
    }
    const cplx<R> k1 = toep_K<R>(a, parts, u);
    const cplx<R> k2 = toep_K<R>(a, parts, w);
    const R h = scale * R(0.5);
    out[q] = mk<R>((k1.x + k2.x) * h, (k1.y - k2.y) * h);
  }
}

}  // namespace tkbn

namespace tkbn_host {

using namespace tkbn;

int toep_assemble(int dtype, int ndim, const int64_t* im_size, const void* parts, double scale, void* out,
                  cudaStream_t s) {
  if (ndim < 1 || ndim > 3) return set_error(TKBN_ERR_UNSUPPORTED, "ndim must be 1, 2 or 3 (got %d)", ndim);
  if (!im_size || !parts || !out) return set_error(TKBN_ERR_INVALID, "null argument");
  ToepAsm a;
  a.nd = ndim;
  a.pstride = 1;
  int64_t total = 1;
  for (int d = 0; d < 3; ++d) {
    a.N[d] = 1;
    if (d < ndim) {
      if (im_size[d] < 1 || im_size[d] > (1 << 23)) return set_error(TKBN_ERR_INVALID, "bad im_size[%d]", d);
      a.N[d] = (int)im_size[d];
      a.pstride *= a.N[d];
      total *= 2 * a.N[d];
    }
  }
  int64_t blocks = (total + 255) / 256;
  if (blocks > 152 * 16) blocks = 152 * 16;
  if (dtype == TKBN_C64)
    k_toep_assemble<float><<<(int)blocks, 256, 0, s>>>(a, (const float2*)parts, (float)scale, (float2*)out);
  else if (dtype == TKBN_C128)
    k_toep_assemble<double><<<(int)blocks, 256, 0, s>>>(a, (const double2*)parts, scale, (double2*)out);
  else
    return set_error(TKBN_ERR_UNSUPPORTED, "unsupported dtype %d", dtype);
  return check_cuda(cudaGetLastError(), "toeplitz assemble launch");
}

}  // namespace tkbn_host
