// Fused 2D FFT passes (fft2d.cu): types shared with the FFT-stage host code.
#pragma once

#include "tkbn_common.cuh"

namespace tkbn {

constexpr int kFftF = 4;             // transforms side by side in one CTA
constexpr int kFftMaxThreads = 512;  // CTA size cap (threads per transform * kFftF)
constexpr int kFftMaxN = 2048;       // largest transform size done in shared memory

// One 1D transform size: nst stages of radix rad[s] (product n); P threads
// per transform (the busiest stage's butterflies, capped by the CTA size).
struct FftPlan1 {
  int n;
  int nst;
  int rad[4];
  int P;
};

struct Fft2dShape {
  int N0, N1;  // image size
  int K0, K1;  // grid size
};

}  // namespace tkbn

namespace tkbn_host {

// Both dims of a 2D grid, with device twiddle tables exp(-2 pi i m / K_d).
struct Fft2d {
  tkbn::Fft2dShape s;
  tkbn::FftPlan1 p0, p1;
  void* tw0;
  void* tw1;
};

// Radix plan for size n; false when n has a prime factor above 5 or needs
// more than 4 stages or more shared memory than a CTA has.
bool fft1_plan(int n, tkbn::FftPlan1* pl);
// cudaMalloc'd table of exp(-2 pi i m / n), m < n (complex64 or complex128).
int fft1_twiddles(int n, bool dbl, void** dev);
// Shared memory of the largest pass for this shape, in bytes.
size_t fft2d_smem(const Fft2d& p, bool dbl);

// grid[b, c] = FFT2(pad(image [* smaps] * scaling) * scale)
int fft2d_forward(const Fft2d& p, int dtype, int64_t B, int64_t C, int64_t ci, const void* image, const void* smaps,
                  int64_t sb, const void* scaling, double scale, void* grid, cudaStream_t st);
// out = [sum_c conj(smaps) *] conj(scaling) * scale * crop(IFFT2(grid)); grid is overwritten
int fft2d_inverse(const Fft2d& p, int dtype, int64_t B, int64_t C, void* grid, const void* smaps, int64_t sb,
                  const void* scaling, double scale, void* out, cudaStream_t st);
// out = [sum_c conj(smaps) *] crop(IFFT2(kernel * scale * FFT2(pad([smaps *] image) * scale)))
int fft2d_toeplitz(const Fft2d& p, int dtype, int64_t B, int64_t C, int64_t ci, const void* image,
                   const void* kernel, int64_t kbatch, int by_channel, const void* smaps, int64_t sb, double scale,
                   void* grid, void* out, cudaStream_t st);

}  // namespace tkbn_host
