// K2 / K5 / K6: FFT stages of the NUFFT and the Toeplitz normal operator,
// fused around cuFFT.
//
//   K2 pad_scale : grid = pad(image [* smaps] * scaling) [* 1/sqrt(prod K)]
//                  (fft_and_scale, torchkbnufft/_nufft/fft.py:35-76, with the
//                  SENSE multiply of modules/kbnufft.py:182-183 folded in)
//   cuFFT        : in-place C2C/Z2Z, forward or inverse, unnormalised
//   K5 crop_scale: image = [sum_c conj(smaps) *] conj(scaling) * crop(grid)
//                  (ifft_and_scale, torchkbnufft/_nufft/fft.py:79-118, with the
//                  coil sum of modules/kbnufft.py:404-405 folded in)
//   K6 kernel_mul: grid *= kernel (fft_filter, torchkbnufft/_nufft/fft.py:121-173)
//
// "ortho" scales by 1/sqrt(prod K) on each transform; the scale is applied in
// the neighbouring elementwise kernel instead of inside the FFT.

#include <cufft.h>

#include <algorithm>

#include <cmath>
#include <new>

#include "fft2d.cuh"
#include "tkbn_common.cuh"

// A plan is either the fused 2D passes of fft2d.cu (2D grids whose sizes
// factor into radices 2..15 and fit shared memory) or a cuFFT plan. 3D grids
// whose three sizes have compile-time plans get the same passes per
// dimension (fused3) for every stage, and no cuFFT plan.
struct tkbn_fft_plan_s {
  cufftHandle handle;
  int ndim;
  int dtype;
  int64_t n[3];
  int64_t batch;
  bool fused;
  tkbn_host::Fft2d f2;
  bool fused3;
  tkbn_host::Fft3d f3;
};

namespace tkbn {

struct Shape {
  int ndim;
  int N[3];  // image size
  int K[3];  // grid size
  int64_t ntot, gtot;
};

// The elementwise stages work on "units": one chunk of up to kChunk elements
// of one row along the last dim. Each unit decomposes its row index once, so
// the per-element work is a load, a few complex multiplies and a store.
constexpr int kChunk = 1024;
constexpr int kStageThreads = 128;

__host__ __device__ __forceinline__ int64_t chunks_of(int64_t n) { return (n + kChunk - 1) / kChunk; }

// Row q (over the leading dims of the grid, row-major) -> image row index, or
// -1 when the row lies in the zero padding.
__device__ __forceinline__ int64_t grid_row_to_image_row(const Shape& s, int64_t q) {
  int64_t nrow = 0, stride = 1;
  for (int d = s.ndim - 2; d >= 0; --d) {
    const int64_t gd = q % s.K[d];
    q /= s.K[d];
    if (gd >= s.N[d]) return -1;
    nrow += gd * stride;
    stride *= s.N[d];
  }
  return nrow;
}

// Image row p (over the leading dims of the image) -> grid row index.
__device__ __forceinline__ int64_t image_row_to_grid_row(const Shape& s, int64_t p) {
  int64_t grow = 0, stride = 1;
  for (int d = s.ndim - 2; d >= 0; --d) {
    const int64_t nd = p % s.N[d];
    p /= s.N[d];
    grow += nd * stride;
    stride *= s.K[d];
  }
  return grow;
}

// K2. Units over the grid rows of (B, C, K...). image has `ci` channels
// (1 with smaps, C without); smaps has `sb` batch entries (1 or B).
template <typename R>
__global__ void __launch_bounds__(kStageThreads) k_pad_scale(Shape s, int64_t B, int64_t C, int64_t ci,
                                                             const cplx<R>* __restrict__ image,
                                                             const cplx<R>* __restrict__ smaps, int64_t sb,
                                                             const cplx<R>* __restrict__ scaling, R scale,
                                                             cplx<R>* __restrict__ grid) {
  const int KX = s.K[s.ndim - 1], NX = s.N[s.ndim - 1];
  const int64_t nchunk = chunks_of(KX);
  const int64_t rows = s.gtot / KX;  // grid rows per (b, c) plane
  const int64_t units = B * C * rows * nchunk;
  for (int64_t u = blockIdx.x; u < units; u += gridDim.x) {
    const int64_t r = u / nchunk;
    const int x0 = (int)(u - r * nchunk) * kChunk;
    const int x1 = min(KX, x0 + kChunk);
    const int64_t bc = r / rows;
    const int64_t nrow = grid_row_to_image_row(s, r - bc * rows);
    cplx<R>* out = grid + r * KX;
    if (nrow < 0) {
      for (int x = x0 + threadIdx.x; x < x1; x += blockDim.x) out[x] = mk<R>(0, 0);
      continue;
    }
    const int64_t b = bc / C, c = bc - b * C;
    const int64_t n0 = nrow * NX;
    const cplx<R>* im = image + (b * ci + (ci == 1 ? 0 : c)) * s.ntot + n0;
    const cplx<R>* sm = smaps ? smaps + ((sb == 1 ? 0 : b) * C + c) * s.ntot + n0 : nullptr;
    const cplx<R>* sc = scaling ? scaling + n0 : nullptr;
    for (int x = x0 + threadIdx.x; x < x1; x += blockDim.x) {
      cplx<R> v = mk<R>(0, 0);
      if (x < NX) {
        v = im[x];
        if (sm) v = cmul<R>(v, sm[x]);
        if (sc) v = cmul<R>(v, sc[x]);
        v = cscale<R>(v, scale);
      }
      out[x] = v;
    }
  }
}

// K5. Units over the output rows: (B, 1, N...) with smaps, else (B, C, N...).
// A unit is kStageThreads elements of one row (one element per thread, so
// that the coil sum of every element runs in its own thread).
template <typename R>
__global__ void __launch_bounds__(kStageThreads) k_crop_scale(Shape s, int64_t B, int64_t C,
                                                              const cplx<R>* __restrict__ grid,
                                                              const cplx<R>* __restrict__ smaps, int64_t sb,
                                                              const cplx<R>* __restrict__ scaling, R scale,
                                                              cplx<R>* __restrict__ out) {
  const int KX = s.K[s.ndim - 1], NX = s.N[s.ndim - 1];
  const int64_t co = smaps ? 1 : C;
  const int64_t nchunk = (NX + kStageThreads - 1) / kStageThreads;
  const int64_t rows = s.ntot / NX;  // image rows per plane
  const int64_t units = B * co * rows * nchunk;
  for (int64_t u = blockIdx.x; u < units; u += gridDim.x) {
    const int64_t r = u / nchunk;
    const int x0 = (int)(u - r * nchunk) * kStageThreads;
    const int x1 = min(NX, x0 + kStageThreads);
    const int64_t bc = r / rows;
    const int64_t p = r - bc * rows;
    const int64_t n0 = p * NX;
    const int64_t g0 = image_row_to_grid_row(s, p) * KX;
    cplx<R>* o = out + r * NX;
    if (smaps) {
      const int64_t b = bc;
      const cplx<R>* gb = grid + b * C * s.gtot + g0;
      const cplx<R>* sm = smaps + (sb == 1 ? 0 : b) * C * s.ntot + n0;
      for (int x = x0 + threadIdx.x; x < x1; x += blockDim.x) {
        cplx<R> sc = scaling ? cconj<R>(scaling[n0 + x]) : mk<R>(1, 0);
        sc = cscale<R>(sc, scale);
        cplx<R> acc = mk<R>(0, 0);
#pragma unroll 4
        for (int64_t c = 0; c < C; ++c) {
          const cplx<R> v = cmul<R>(gb[c * s.gtot + x], sc);
          acc = cfma<R>(v, cconj<R>(sm[c * s.ntot + x]), acc);
        }
        o[x] = acc;
      }
    } else {
      const cplx<R>* gp = grid + bc * s.gtot + g0;
      for (int x = x0 + threadIdx.x; x < x1; x += blockDim.x) {
        cplx<R> sc = scaling ? cconj<R>(scaling[n0 + x]) : mk<R>(1, 0);
        sc = cscale<R>(sc, scale);
        o[x] = cmul<R>(gp[x], sc);
      }
    }
  }
}

// K6. grid[b, c, g] *= kernel[k, g] * scale with k = 0 (shared kernel), b
// (one kernel per batch item) or c (one kernel per channel: torch
// broadcasting of a (K, *grid) kernel against (B, C, *grid)). Units are
// kChunk-element chunks of one (b, c) plane.
template <typename R>
__global__ void __launch_bounds__(kStageThreads) k_kernel_mul(int64_t gtot, int64_t B, int64_t C,
                                                              const cplx<R>* __restrict__ kernel, int64_t kbatch,
                                                              int by_channel, R scale, cplx<R>* __restrict__ grid) {
  const int64_t nchunk = chunks_of(gtot);
  const int64_t units = B * C * nchunk;
  for (int64_t u = blockIdx.x; u < units; u += gridDim.x) {
    const int64_t bc = u / nchunk;
    const int64_t g0 = (u - bc * nchunk) * kChunk;
    const int n = (int)min((int64_t)kChunk, gtot - g0);
    const int64_t k = kbatch == 1 ? 0 : (by_channel ? bc % C : bc / C);
    cplx<R>* gp = grid + bc * gtot + g0;
    const cplx<R>* kp = kernel + k * gtot + g0;
    for (int x = threadIdx.x; x < n; x += blockDim.x) gp[x] = cscale<R>(cmul<R>(gp[x], kp[x]), scale);
  }
}

}  // namespace tkbn

TKBN_DEFINE_STATUS_READER(status_fft)

namespace tkbn_host {

using namespace tkbn;

// Blocks for `units` work units: at most 16 resident 128-thread blocks on
// each of the 152 SMs, the rest taken by the grid-stride loop.
static int stage_blocks(int64_t units) {
  int64_t b = units;
  if (b > 152 * 16) b = 152 * 16;
  if (b < 1) b = 1;
  return (int)b;
}

static int check_cufft(cufftResult r, const char* what) {
  if (r == CUFFT_SUCCESS) return TKBN_OK;
  return set_error(TKBN_ERR_CUFFT, "%s: cuFFT error %d", what, (int)r);
}

int fft_plan_create(const tkbn_geometry* g, int64_t B, int64_t C, tkbn_fft_plan* out) {
  if (!g || !out) return set_error(TKBN_ERR_INVALID, "null argument");
  if (g->ndim < 1 || g->ndim > 3) return set_error(TKBN_ERR_UNSUPPORTED, "ndim must be 1, 2 or 3");
  if (g->dtype != TKBN_C64 && g->dtype != TKBN_C128) return set_error(TKBN_ERR_UNSUPPORTED, "unsupported dtype");
  if (B < 1 || C < 1) return set_error(TKBN_ERR_INVALID, "batch and coil counts must be >= 1");
  tkbn_fft_plan p = new (std::nothrow) tkbn_fft_plan_s();
  if (!p) return set_error(TKBN_ERR_INVALID, "out of host memory");
  p->ndim = g->ndim;
  p->dtype = g->dtype;
  p->batch = B * C;
  long long n[3];
  for (int d = 0; d < g->ndim; ++d) {
    n[d] = g->grid_size[d];
    p->n[d] = g->grid_size[d];
  }
  p->fused = false;
  p->fused3 = false;
  if (g->ndim == 3) {
    int K[3] = {(int)g->grid_size[0], (int)g->grid_size[1], (int)g->grid_size[2]};
    const bool dbl = g->dtype == TKBN_C128;
    // the largest pass: a column pass of 8 columns or a row pass of 4 rows (plus the coil sum row)
    size_t smem = 0;
    for (int d = 0; d < 3; ++d) {
      const size_t e = dbl ? 16 : 8;
      const size_t c = 2 * (size_t)K[d] * 8 * e, r = (2 * (size_t)K[d] * tkbn::kFftF + (size_t)K[d]) * e;
      smem = std::max(smem, std::max(c, r));
    }
    if (fft3d_supported(K) && smem <= 200 * 1024) {
      int rc = TKBN_OK;
      for (int d = 0; d < 3; ++d) p->f3.tw[d] = nullptr;
      for (int d = 0; d < 3 && !rc; ++d) {
        p->f3.K[d] = K[d];
        rc = fft1_twiddles(K[d], dbl, &p->f3.tw[d]);
      }
      if (rc) {
        for (int d = 0; d < 3; ++d) cudaFree(p->f3.tw[d]);
        delete p;
        return rc;
      }
      p->fused3 = true;  // every 3D stage runs on the fused passes: no cuFFT plan
      *out = p;
      return TKBN_OK;
    }
  }
  if (g->ndim == 2 && g->grid_size[0] <= tkbn::kFftMaxN && g->grid_size[1] <= tkbn::kFftMaxN &&
      fft1_plan((int)g->grid_size[0], &p->f2.p0) && fft1_plan((int)g->grid_size[1], &p->f2.p1)) {
    p->f2.s.K0 = (int)g->grid_size[0];
    p->f2.s.K1 = (int)g->grid_size[1];
    p->f2.s.N0 = p->f2.s.K0;
    p->f2.s.N1 = p->f2.s.K1;
    const bool dbl = g->dtype == TKBN_C128;
    if (fft2d_smem(p->f2, dbl) <= 200 * 1024) {
      p->f2.tw0 = p->f2.tw1 = nullptr;
      int rc = fft1_twiddles(p->f2.s.K0, dbl, &p->f2.tw0);
      if (!rc) rc = fft1_twiddles(p->f2.s.K1, dbl, &p->f2.tw1);
      if (rc) {
        cudaFree(p->f2.tw0);
        cudaFree(p->f2.tw1);
        delete p;
        return rc;
      }
      p->fused = true;
      *out = p;
      return TKBN_OK;
    }
  }
  int rc = check_cufft(cufftCreate(&p->handle), "cufftCreate");
  if (rc) {
    delete p;
    return rc;
  }
  size_t work = 0;
  rc = check_cufft(cufftMakePlanMany64(p->handle, g->ndim, n, nullptr, 1, 0, nullptr, 1, 0,
                                       g->dtype == TKBN_C64 ? CUFFT_C2C : CUFFT_Z2Z, (long long)p->batch, &work),
                   "cufftMakePlanMany64");
  if (rc) {
    cufftDestroy(p->handle);
    delete p;
    return rc;
  }
  *out = p;
  return TKBN_OK;
}

int fft_plan_destroy(tkbn_fft_plan p) {
  if (!p) return TKBN_OK;
  int rc;
  if (p->fused) {
    rc = check_cuda(cudaFree(p->f2.tw0), "free twiddles");
    const int rc1 = check_cuda(cudaFree(p->f2.tw1), "free twiddles");
    if (!rc) rc = rc1;
  } else if (p->fused3) {
    rc = TKBN_OK;
    for (int d = 0; d < 3; ++d) {
      const int rc1 = check_cuda(cudaFree(p->f3.tw[d]), "free twiddles");
      if (!rc) rc = rc1;
    }
  } else {
    rc = check_cufft(cufftDestroy(p->handle), "cufftDestroy");
  }
  delete p;
  return rc;
}

// The fused passes of a plan with this call's image size.
static Fft2d fused_for(const tkbn_fft_plan p, const Shape& s) {
  Fft2d f = p->f2;
  f.s = tkbn::fft2d_shape(s.N[0], s.N[1], f.s.K0, f.s.K1);
  return f;
}

static Fft3d fused3_for(const tkbn_fft_plan p, const Shape& s) {
  Fft3d f = p->f3;
  for (int d = 0; d < 3; ++d) f.N[d] = s.N[d];
  return f;
}

static int check_plan(const tkbn_geometry* g, tkbn_fft_plan p, int64_t B, int64_t C) {
  if (!p) return set_error(TKBN_ERR_INVALID, "fft plan is null");
  if (p->ndim != g->ndim || p->dtype != g->dtype || p->batch != B * C)
    return set_error(TKBN_ERR_INVALID, "fft plan does not match geometry/batch");
  for (int d = 0; d < g->ndim; ++d)
    if (p->n[d] != g->grid_size[d]) return set_error(TKBN_ERR_INVALID, "fft plan does not match grid size");
  return TKBN_OK;
}

int fft_exec(tkbn_fft_plan p, void* data, int direction, cudaStream_t s) {
  int rc = check_cufft(cufftSetStream(p->handle, s), "cufftSetStream");
  if (rc) return rc;
  if (p->dtype == TKBN_C64)
    return check_cufft(cufftExecC2C(p->handle, (cufftComplex*)data, (cufftComplex*)data, direction), "cufftExecC2C");
  return check_cufft(cufftExecZ2Z(p->handle, (cufftDoubleComplex*)data, (cufftDoubleComplex*)data, direction),
                     "cufftExecZ2Z");
}

static int make_shape(const tkbn_geometry* g, Shape* s) {
  s->ndim = g->ndim;
  s->ntot = 1;
  s->gtot = 1;
  for (int d = 0; d < 3; ++d) {
    s->N[d] = d < g->ndim ? (int)g->im_size[d] : 1;
    s->K[d] = d < g->ndim ? (int)g->grid_size[d] : 1;
  }
  for (int d = 0; d < g->ndim; ++d) {
    if (g->im_size[d] < 1 || g->grid_size[d] < g->im_size[d])
      return set_error(TKBN_ERR_INVALID, "grid_size must be >= im_size in every dimension");
    s->ntot *= g->im_size[d];
    s->gtot *= g->grid_size[d];
  }
  return TKBN_OK;
}

static double ortho_scale(const Shape& s, int norm) { return norm == TKBN_NORM_ORTHO ? 1.0 / std::sqrt((double)s.gtot) : 1.0; }

template <typename R>
static int pad_scale_r(const Shape& s, int64_t B, int64_t C, int64_t ci, const void* image, const void* smaps,
                       int64_t sb, const void* scaling, double scale, void* grid, cudaStream_t st) {
  const int64_t kx = s.K[s.ndim - 1];
  const int blocks = stage_blocks(B * C * (s.gtot / kx) * chunks_of(kx));
  k_pad_scale<R><<<blocks, kStageThreads, 0, st>>>(s, B, C, ci, (const cplx<R>*)image, (const cplx<R>*)smaps, sb,
                                                   (const cplx<R>*)scaling, (R)scale, (cplx<R>*)grid);
  return check_cuda(cudaGetLastError(), "pad_scale launch");
}

template <typename R>
static int crop_scale_r(const Shape& s, int64_t B, int64_t C, const void* grid, const void* smaps, int64_t sb,
                        const void* scaling, double scale, void* out, cudaStream_t st) {
  const int64_t co = smaps ? 1 : C;
  const int64_t nx = s.N[s.ndim - 1];
  const int blocks = stage_blocks(B * co * (s.ntot / nx) * ((nx + kStageThreads - 1) / kStageThreads));
  k_crop_scale<R><<<blocks, kStageThreads, 0, st>>>(s, B, C, (const cplx<R>*)grid, (const cplx<R>*)smaps, sb,
                                                    (const cplx<R>*)scaling, (R)scale, (cplx<R>*)out);
  return check_cuda(cudaGetLastError(), "crop_scale launch");
}

int fft_and_scale(const tkbn_geometry* g, tkbn_fft_plan plan, const void* image, const void* smaps,
                  int64_t smaps_batch, const void* scaling, int64_t B, int64_t C, int norm, void* grid,
                  cudaStream_t st) {
  Shape s;
  int rc = make_shape(g, &s);
  if (rc || (rc = check_plan(g, plan, B, C))) return rc;
  if (!image || !grid) return set_error(TKBN_ERR_INVALID, "null image or grid");
  if (smaps && smaps_batch != 1 && smaps_batch != B) return set_error(TKBN_ERR_INVALID, "smaps batch must be 1 or B");
  if (norm != TKBN_NORM_NONE && norm != TKBN_NORM_ORTHO) return set_error(TKBN_ERR_INVALID, "Only option for norm is 'ortho'.");
  const int64_t ci = smaps ? 1 : C;
  const double sc = ortho_scale(s, norm);
  if (plan->fused)
    return fft2d_forward(fused_for(plan, s), g->dtype, B, C, ci, image, smaps, smaps_batch, scaling, sc, grid, st);
  if (plan->fused3)
    return fft3d_forward(fused3_for(plan, s), g->dtype, B, C, ci, image, smaps, smaps_batch, scaling, sc, grid, st);
  rc = g->dtype == TKBN_C64 ? pad_scale_r<float>(s, B, C, ci, image, smaps, smaps_batch, scaling, sc, grid, st)
                            : pad_scale_r<double>(s, B, C, ci, image, smaps, smaps_batch, scaling, sc, grid, st);
  if (rc) return rc;
  return fft_exec(plan, grid, CUFFT_FORWARD, st);
}

int ifft_and_scale(const tkbn_geometry* g, tkbn_fft_plan plan, void* grid, const void* smaps, int64_t smaps_batch,
                   const void* scaling, int64_t B, int64_t C, int norm, void* image, cudaStream_t st) {
  Shape s;
  int rc = make_shape(g, &s);
  if (rc || (rc = check_plan(g, plan, B, C))) return rc;
  if (!image || !grid) return set_error(TKBN_ERR_INVALID, "null image or grid");
  if (smaps && smaps_batch != 1 && smaps_batch != B) return set_error(TKBN_ERR_INVALID, "smaps batch must be 1 or B");
  if (norm != TKBN_NORM_NONE && norm != TKBN_NORM_ORTHO) return set_error(TKBN_ERR_INVALID, "Only option for norm is 'ortho'.");
  const double sc = ortho_scale(s, norm);
  if (plan->fused)
    return fft2d_inverse(fused_for(plan, s), g->dtype, B, C, grid, smaps, smaps_batch, scaling, sc, image, st);
  if (plan->fused3)
    return fft3d_inverse(fused3_for(plan, s), g->dtype, B, C, grid, smaps, smaps_batch, scaling, sc, image, st);
  rc = fft_exec(plan, grid, CUFFT_INVERSE, st);
  if (rc) return rc;
  return g->dtype == TKBN_C64 ? crop_scale_r<float>(s, B, C, grid, smaps, smaps_batch, scaling, sc, image, st)
                              : crop_scale_r<double>(s, B, C, grid, smaps, smaps_batch, scaling, sc, image, st);
}

int toep_apply(const tkbn_geometry* g, tkbn_fft_plan plan, const void* image, const void* kernel, int64_t kbatch,
               int by_channel, const void* smaps, int64_t smaps_batch, int64_t B, int64_t C, int norm, void* grid,
               void* out, cudaStream_t st) {
  Shape s;
  int rc = make_shape(g, &s);
  if (rc || (rc = check_plan(g, plan, B, C))) return rc;
  if (!image || !kernel || !grid || !out) return set_error(TKBN_ERR_INVALID, "null pointer argument");
  if (!by_channel && kbatch != 1 && kbatch != B)
    return set_error(TKBN_ERR_INVALID, "If using batch dimension, kernel must have same batch size as image");
  if (by_channel && kbatch != 1 && kbatch != C)
    return set_error(TKBN_ERR_INVALID, "kernel batch must be 1 or the channel count");
  if (smaps && smaps_batch != 1 && smaps_batch != B) return set_error(TKBN_ERR_INVALID, "smaps batch must be 1 or B");
  if (norm != TKBN_NORM_NONE && norm != TKBN_NORM_ORTHO) return set_error(TKBN_ERR_INVALID, "Only option for norm is 'ortho'.");
  const double sc = ortho_scale(s, norm);
  const int64_t ci = smaps ? 1 : C;
  if (plan->fused3)
    return fft3d_toeplitz(fused3_for(plan, s), g->dtype, B, C, ci, image, kernel, kbatch, by_channel, smaps,
                          smaps_batch, sc, grid, out, st);
  if (plan->fused)
    return fft2d_toeplitz(fused_for(plan, s), g->dtype, B, C, ci, image, kernel, kbatch, by_channel, smaps,
                          smaps_batch, sc, grid, out, st);
  if (g->dtype == TKBN_C64) {
    if ((rc = pad_scale_r<float>(s, B, C, ci, image, smaps, smaps_batch, nullptr, sc, grid, st))) return rc;
    if ((rc = fft_exec(plan, grid, CUFFT_FORWARD, st))) return rc;
    k_kernel_mul<float><<<stage_blocks(B * C * chunks_of(s.gtot)), kStageThreads, 0, st>>>(
        s.gtot, B, C, (const float2*)kernel, kbatch, by_channel, (float)sc, (float2*)grid);
    if ((rc = check_cuda(cudaGetLastError(), "kernel_mul launch"))) return rc;
    if ((rc = fft_exec(plan, grid, CUFFT_INVERSE, st))) return rc;
    return crop_scale_r<float>(s, B, C, grid, smaps, smaps_batch, nullptr, 1.0, out, st);
  }
  if ((rc = pad_scale_r<double>(s, B, C, ci, image, smaps, smaps_batch, nullptr, sc, grid, st))) return rc;
  if ((rc = fft_exec(plan, grid, CUFFT_FORWARD, st))) return rc;
  k_kernel_mul<double><<<stage_blocks(B * C * chunks_of(s.gtot)), kStageThreads, 0, st>>>(
      s.gtot, B, C, (const double2*)kernel, kbatch, by_channel, sc, (double2*)grid);
  if ((rc = check_cuda(cudaGetLastError(), "kernel_mul launch"))) return rc;
  if ((rc = fft_exec(plan, grid, CUFFT_INVERSE, st))) return rc;
  return crop_scale_r<double>(s, B, C, grid, smaps, smaps_batch, nullptr, 1.0, out, st);
}

}  // namespace tkbn_host
