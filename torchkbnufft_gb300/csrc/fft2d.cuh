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
  // Row passes: image row n0 sits in grid row (n0 / ny) * ky + n0 % ny (a 3D
  // volume's (z, y) rows: ny = Ny, ky = Ky; 2D: ny = N0). Column passes: unit
  // plane p is grid plane (p / pk) * pt + p % pk (the nonzero z slices of a
  // 3D volume: pk = Nz, pt = Kz; 2D: pk = pt = 1).
  int ny, ky;
  int pk, pt;
};

// The fused-pass shape of a 2D grid (every mapping the identity).
inline Fft2dShape fft2d_shape(int N0, int N1, int K0, int K1) {
  Fft2dShape s;
  s.N0 = N0;
  s.N1 = N1;
  s.K0 = K0;
  s.K1 = K1;
  s.ny = N0 > 0 ? N0 : 1;
  s.ky = K0;
  s.pk = s.pt = 1;
  return s;
}

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
// 3D grids whose three sizes have compile-time plans: the same passes per
// dimension, skipping the zero padding (rows past Nx in x, rows past Ny and
// slices past Nz never read), with twiddles per dim.
struct Fft3d {
  int N[3], K[3];
  void* tw[3];
};
bool fft3d_supported(const int K[3]);
// grid[b, c] = FFT3(pad(image [* smaps] * scaling) * scale)
int fft3d_forward(const Fft3d& p, int dtype, int64_t B, int64_t C, int64_t ci, const void* image, const void* smaps,
                  int64_t sb, const void* scaling, double scale, void* grid, cudaStream_t st);
// out = [sum_c conj(smaps) *] conj(scaling) * scale * crop(IFFT3(grid)); grid is overwritten
int fft3d_inverse(const Fft3d& p, int dtype, int64_t B, int64_t C, void* grid, const void* smaps, int64_t sb,
                  const void* scaling, double scale, void* out, cudaStream_t st);
// out = [sum_c conj(smaps) *] crop(IFFT3(kernel * scale * FFT3(pad([smaps *] image) * scale)))
int fft3d_toeplitz(const Fft3d& p, int dtype, int64_t B, int64_t C, int64_t ci, const void* image,
                   const void* kernel, int64_t kbatch, int by_channel, const void* smaps, int64_t sb, double scale,
                   void* grid, void* out, cudaStream_t st);
// out = [sum_c conj(smaps) *] crop(IFFT2(kernel * scale * FFT2(pad([smaps *] image) * scale)))
int fft2d_toeplitz(const Fft2d& p, int dtype, int64_t B, int64_t C, int64_t ci, const void* image,
                   const void* kernel, int64_t kbatch, int by_channel, const void* smaps, int64_t sb, double scale,
                   void* grid, void* out, cudaStream_t st);

}  // namespace tkbn_host
