// Shared device helpers for the sm_103a table-mode KB NUFFT kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/tkbn_gb300.h"

namespace tkbn {

// Entries of a tile's point list staged per adjoint batch (2D register adjoint).
constexpr int kListChunk = 256;
// floats per sorted point of the 3D linear-phase factor records
constexpr int kLp3PRec = 24;

constexpr int kMaxDim = 3;
constexpr int kMaxJ = 8;  // numpoints supported per dimension

// Device status bits (OR-ed into g_status by kernels whose own checks fail).
constexpr int kStatusNonFinite = 1;     // a trajectory coordinate was NaN/Inf or out of range
constexpr int kStatusOutsidePatch = 2;  // a point's footprint left its tile patch (layout mismatch)
constexpr int kStatusBadItem = 4;       // malformed work item

// One status word per translation unit (static linkage, no relocatable device
// code needed); each unit exposes a host reader, see TKBN_DEFINE_STATUS_READER.
static __device__ int g_status;

// ---------------------------------------------------------------- complex
template <typename R>
struct Cplx;
template <>
struct Cplx<float> {
  using T = float2;
};
template <>
struct Cplx<double> {
  using T = double2;
};
template <typename R>
using cplx = typename Cplx<R>::T;

template <typename R>
__host__ __device__ __forceinline__ cplx<R> mk(R re, R im) {
  cplx<R> z;
  z.x = re;
  z.y = im;
  return z;
}
template <typename R>
__device__ __forceinline__ cplx<R> cmul(cplx<R> a, cplx<R> b) {
  return mk<R>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// a * conj(b)
template <typename R>
__device__ __forceinline__ cplx<R> cmulc(cplx<R> a, cplx<R> b) {
  return mk<R>(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}
// acc + a * b
template <typename R>
__device__ __forceinline__ cplx<R> cfma(cplx<R> a, cplx<R> b, cplx<R> acc) {
  acc.x = fma(a.x, b.x, acc.x);
  acc.x = fma(-a.y, b.y, acc.x);
  acc.y = fma(a.x, b.y, acc.y);
  acc.y = fma(a.y, b.x, acc.y);
  return acc;
}
// acc + conj(a) * b
template <typename R>
__device__ __forceinline__ cplx<R> cfmac(cplx<R> a, cplx<R> b, cplx<R> acc) {
  acc.x = fma(a.x, b.x, acc.x);
  acc.x = fma(a.y, b.y, acc.x);
  acc.y = fma(a.x, b.y, acc.y);
  acc.y = fma(-a.y, b.x, acc.y);
  return acc;
}
template <typename R>
__device__ __forceinline__ cplx<R> cscale(cplx<R> a, R s) {
  return mk<R>(a.x * s, a.y * s);
}
template <typename R>
__device__ __forceinline__ cplx<R> cconj(cplx<R> a) {
  return mk<R>(a.x, -a.y);
}

// Correctly rounded single operations, never contracted into FMAs. The
// reference evaluates these steps as separate tensor ops, so each result is
// rounded on its own; matching that keeps table-bin selection bit-identical.
__device__ __forceinline__ float sub_rn(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ double sub_rn(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float add_rn(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double add_rn(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ float div_rn(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ double div_rn(double a, double b) { return __ddiv_rn(a, b); }
__device__ __forceinline__ void sincos_acc(float x, float* s, float* c) { sincosf(x, s, c); }
__device__ __forceinline__ void sincos_acc(double x, double* s, double* c) { sincos(x, s, c); }

// ---------------------------------------------------------------- geometry
// Per-launch constants for interpolation kernels (passed by value).
template <typename R>
struct Geo {
  int ndim;
  int K[kMaxDim];        // grid size
  int J[kMaxDim];        // numpoints
  int L[kMaxDim];        // table oversampling
  int center[kMaxDim];   // floor(J*L/2)
  int tmax[kMaxDim];     // last valid table index (J*L)
  int T[kMaxDim];        // tile edge (cells)
  int P[kMaxDim];        // patch extent T + J - 1
  int ntile[kMaxDim];    // tiles per dim
  int ntiles;            // prod ntile
  R gam[kMaxDim];        // fl(fl(1/K) * fl(2 pi))
  R halfJ[kMaxDim];      // J / 2
  R Lr[kMaxDim];         // L as R
  R nshift[kMaxDim];
  const cplx<R>* tab[kMaxDim];
  const cplx<R>* dtab[kMaxDim];
  bool half[kMaxDim];    // table read through its conjugate symmetry (J*L even)
};

// Work item of the sorted layout: points [start, start+len) of tile `key`.
struct Item {
  int key;
  int start;
  int len;
  int pad;
};

// Positive modulo.
__device__ __forceinline__ int pmod(int a, int k) {
  int r = a % k;
  return r < 0 ? r + k : r;
}

// a mod k for a within one period of [0, k) (the usual case: one compare and
// add), falling back to the general modulo otherwise.
__device__ __forceinline__ int wrap_cell(int a, int k) {
  int w = a < 0 ? a + k : (a >= k ? a - k : a);
  if ((unsigned)w >= (unsigned)k) w = pmod(a, k);
  return w;
}

// Tiles whose points can reach an output tile: per dim, the tile itself and
// up to nsrc-1 tiles before it (periodic). ncombo = prod nsrc.
struct SrcSpan {
  int nsrc[kMaxDim];
  int ncombo;
};

// Linear tile index (within one trajectory) of source combination `combo`
// for the output tile with per-dim tile coordinates td.
template <typename R>
__device__ __forceinline__ int source_tile(const Geo<R>& geo, const SrcSpan& span, const int* td, int combo) {
  int rest = combo;
  int sd[kMaxDim] = {0, 0, 0};
#pragma unroll
  for (int d = kMaxDim - 1; d >= 0; --d) {
    if (d < geo.ndim) {
      const int delta = rest % span.nsrc[d];
      rest /= span.nsrc[d];
      int s = td[d] - delta;
      if (s < 0) s += geo.ntile[d];
      sd[d] = s;
    }
  }
  int key = 0;
#pragma unroll
  for (int d = 0; d < kMaxDim; ++d)
    if (d < geo.ndim) key = key * geo.ntile[d] + sd[d];
  return key;
}

// First neighbour index of a point along one dimension: 1 + floor(tm - J/2),
// with tm = omega / gam (torchkbnufft/_nufft/interp.py:171, 177). Returns
// false for coordinates that are not finite or far outside any grid.
template <typename R>
__device__ __forceinline__ bool base_index(R om, R gam, R halfJ, R* tm_out, int* base_out) {
  R tm = div_rn(om, gam);
  R f = floor(sub_rn(tm, halfJ));
  *tm_out = tm;
  if (!(fabs(f) < R(1 << 30))) {
    *base_out = 0;
    return false;
  }
  *base_out = 1 + (int)f;
  return true;
}

// Table bin for the neighbour at cell g: round_half_even((tm - g) * L) + center
// (torchkbnufft/_nufft/interp.py:129-132), clamped to the table.
template <typename R>
__device__ __forceinline__ int table_bin(R tm, int g, R Lr, int center, int tmax) {
  R s = mul_rn(sub_rn(tm, (R)g), Lr);
  int k = (int)rint(s) + center;
  return min(max(k, 0), tmax);
}

// Table entry k. The tabulated kernel is KB(u) exp(-i r u) at u = k/L - J/2
// with KB even, so entry center + d is the conjugate of entry center - d
// (exactly, when J*L is even): only the first half of the table is read, which
// halves its cache footprint. `half` selects this mode.
template <typename R>
__device__ __forceinline__ cplx<R> table_entry(const cplx<R>* __restrict__ tab, int k, int center, bool half) {
  if (half && k > center) {
    const cplx<R> v = __ldg(&tab[2 * center - k]);
    return mk<R>(v.x, -v.y);
  }
  return __ldg(&tab[k]);
}

// fftshift phase argument sum_d omega_d * n_shift_d with each product rounded
// before the sum (torchkbnufft/_nufft/interp.py:200-203).
template <typename R, int D>
__device__ __forceinline__ R phase_arg(const R* om, const R* nshift) {
  R a = mul_rn(om[0], nshift[0]);
#pragma unroll
  for (int d = 1; d < D; ++d) a = add_rn(a, mul_rn(om[d], nshift[d]));
  return a;
}

}  // namespace tkbn

// Host-side helpers shared by the .cu files.
namespace tkbn_host {

int set_error(int code, const char* fmt, ...);
int check_cuda(cudaError_t e, const char* what);
// CTAs of `kernel` that fit on the whole GPU at once (per-SM occupancy times
// the SM count) with `threads` threads and `smem` bytes of dynamic shared
// memory, raising the kernel's shared-memory limit first. Cached per
// (device, kernel, threads, smem): after the first call it makes no CUDA
// call, so it is cheap on every launch and safe inside stream capture.
int resident_grid(const void* kernel, int threads, size_t smem, int64_t* blocks);

// Byte layout of the sorted-point workspace.
struct PointsLayout {
  int64_t nkeys;       // ntraj * ntiles
  int64_t npts_total;  // ntraj * M
  int64_t max_items;   // upper bound on work items
  int key_bits;
  int item_key_bits;
  int tile[3];
  int ntile[3];
  int chunk;
  tkbn::SrcSpan span;   // source tiles of an output tile (adjoint)
  bool owned_ok;        // every K_d >= T_d + J_d - 1: a footprint meets a tile in one contiguous run
  int adj_chunk;        // max candidates per adjoint sub-job
  int64_t max_subjobs;  // upper bound on adjoint sub-jobs
  int sj_key_bits;
  // 2D owned tiles: per output tile, the list of points whose footprint
  // reaches it ({sorted index, m, row offset, column offset}), built once
  // per trajectory; the adjoint's sub-jobs are ranges of these lists.
  bool vlist;
  int64_t max_valid;  // upper bound on list entries (ncombo * npts_total)
  // Footprint start of a list entry in the last two dims:
  // k = (rx + Jc - 1) * kny + (ry + Jr - 1), k < knk.
  //  * 3D (ksort): each tile's list is sorted by start (stable); the entries
  //    of one start are a run and koff[tile][k] is its first entry
  //    (koff[tile][knk] = end).
  //  * 2D complex64 J = 6 16 x 14 layouts (csort): the list keeps its order
  //    (source tile, then sorted point order: runs of consecutive m), and
  //    vsort holds each kListChunk-entry chunk of it sorted by start, entry
  //    {sorted index, position in the chunk, ry, rx}; koff row
  //    (voff[tile] + first) / kListChunk + tile holds the chunk's run starts.
  bool ksort, csort;
  int kny, knk;
  int64_t koff_rows;
  // csort layouts: room for each sorted point's 12 conjugated table factors,
  // filled by the register adjoint before it runs
  bool pfac;
  // 3D chunk-sorted layouts: list of points the linear-phase adjoint leaves
  // out (count first, then indices), and room for each sorted point's 18
  // real table magnitudes and phase word (24 floats), filled by a pre-pass
  bool lfix;
  bool pfac3;
  size_t off_pfac3;
  size_t off_hdr, off_keys_in, off_vals_in, off_keys, off_vals, off_counts, off_tile_off, off_nit, off_item_off,
      off_items, off_items_raw, off_ikeys_in, off_ikeys, off_ivals_in, off_ivals, off_coords, off_phase,
      off_tile_work, off_tile_nsub, off_tile_suboff, off_sj_raw, off_adj_jobs, off_sj_keys_in, off_sj_keys,
      off_sj_vals_in, off_sj_vals, off_vcount, off_voff, off_vlist, off_vtmp, off_vsort, off_koff, off_pfac, off_lfix, off_cub;
  size_t cub_bytes;
  size_t total;
};

int points_layout(const tkbn_geometry* g, const tkbn_points_desc* p, PointsLayout* out);

// Default tile edge and chunk per dimension count.
void default_tiles(const tkbn_geometry* g, int tile[3], int* chunk);

// Per-unit status readers (read and clear; synchronise the stream).
int status_points(cudaStream_t s, int* st);
int status_interp(cudaStream_t s, int* st);
int status_fft(cudaStream_t s, int* st);

}  // namespace tkbn_host

#define TKBN_DEFINE_STATUS_READER(NAME)                                                   \
  namespace tkbn_host {                                                                    \
  int NAME(cudaStream_t s, int* st) {                                                      \
    int v = 0;                                                                             \
    int rc = check_cuda(cudaMemcpyFromSymbolAsync(&v, tkbn::g_status, sizeof(int), 0,     \
                                                  cudaMemcpyDeviceToHost, s),              \
                        "read status");                                                    \
    if (rc) return rc;                                                                     \
    rc = check_cuda(cudaStreamSynchronize(s), "sync for status");                         \
    if (rc) return rc;                                                                     \
    const int zero = 0;                                                                    \
    rc = check_cuda(cudaMemcpyToSymbolAsync(tkbn::g_status, &zero, sizeof(int), 0,         \
                                            cudaMemcpyHostToDevice, s),                    \
                    "clear status");                                                       \
    if (rc) return rc;                                                                     \
    rc = check_cuda(cudaStreamSynchronize(s), "sync for status");                         \
    *st |= v;                                                                              \
    return rc;                                                                             \
  }                                                                                        \
  }
