// cube_pk.cu -- the matter power spectrum of the resident particles on the
// device: the CIC density of cicpower.f90:100-133 (mass 1, position
// (cell + frac)*ng/nc - 0.5), its density contrast (:171-176), and the binned
// auto/cross power of powerspectrum.f90:cross_power (:21-135) with linear bins
// ibin = nint(|k|), the CIC window 1/sinc^4 and the 4 pi k^3 weight.
//
// The mesh buffers of the fine PM are borrowed as scratch (the spectrum is an
// analysis call between steps): force plane 0 holds the particles' density
// and spectrum, plane 1 the optional second field, plane 2 the per-block
// partial sums.  Sums over modes run in FP32 inside a block and in FP64
// across blocks (the reference sums in real(4) throughout).
#include <cmath>
#include <vector>

#include "cube_internal.cuh"

namespace {

constexpr int PK_Q = 7;        // accumulated quantities per bin (xi(1:7))
constexpr int PK_T = 256;

// rho/mean - 1 over the ng^3 interior of a padded mesh (cicpower.f90:171-176)
__global__ void k_pk_delta(float* rho, int ng, float inv_mean) {
  const int64_t rows = (int64_t)ng * ng;
  for (int64_t r = blockIdx.x; r < rows; r += gridDim.x) {
    float* row = rho + r * (ng + 2);
    for (int x = threadIdx.x; x < ng; x += blockDim.x) row[x] = __fmaf_rn(row[x], inv_mean, -1.0f);
  }
}

// One thread per (j, k) row of the half spectrum, walking i = 0..ng/2; |k|
// grows with i along a row, so each thread keeps running sums for its current
// bin and adds them to the block's shared bins when the bin changes.
__global__ void __launch_bounds__(PK_T) k_pk_bin(const float2* __restrict__ c1, const float2* __restrict__ c2, int ng,
                                                 int nbin, float* __restrict__ part) {
  extern __shared__ float sb[];  // PK_Q * nbin
  for (int i = threadIdx.x; i < PK_Q * nbin; i += blockDim.x) sb[i] = 0.f;
  __syncthreads();
  const int nyq = ng / 2, nh = nyq + 1;
  const float inv_n3 = 1.0f / ((float)ng * (float)ng * (float)ng);  // cx=cxyz/ng^3
  const float four_pi = 4.0f * CUBE_PI_F;
  const int64_t rows = (int64_t)ng * ng;
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < rows; r += (int64_t)gridDim.x * blockDim.x) {
    const int j = (int)(r % ng), k = (int)(r / ng);
    const int ky = (j + nyq) % ng - nyq, kz = (k + nyq) % ng - nyq;
    const float sy = ky == 0 ? 1.0f : sinf(CUBE_PI_F * ky / ng) / (CUBE_PI_F * ky / ng);
    const float sz = kz == 0 ? 1.0f : sinf(CUBE_PI_F * kz / ng) / (CUBE_PI_F * kz / ng);
    int cur = -1;
    float acc[PK_Q] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    const int64_t base = r * nh;
    for (int i = 0; i < nh; i++) {
      // powerspectrum.f90:60-62: the zero mode, and the conjugate duplicates on
      // the i = 0 and i = nyquist planes
      const bool edge_i = i == 0 || i == nyq;
      if (i == 0 && j == 0 && k == 0) continue;
      if (edge_i && j > nyq) continue;
      if (edge_i && (j == 0 || j == nyq) && k > nyq) continue;
      const int kx = (i + nyq) % ng - nyq;
      const float kr = sqrtf((float)(kx * kx + ky * ky + kz * kz));
      const float sx = kx == 0 ? 1.0f : sinf(CUBE_PI_F * kx / ng) / (CUBE_PI_F * kx / ng);
      const float s = sx * sy * sz, s2 = s * s, s4 = s2 * s2;
      const int b = (int)roundf(kr) - 1;  // ibin = nint(kr), 1-based
      float2 a = c1[base + i];
      float2 bb = c2[base + i];
      const float w = four_pi * kr * kr * kr / s4 * inv_n3 * inv_n3;
      if (b != cur) {
        if (cur >= 0 && cur < nbin)
          for (int q = 0; q < PK_Q; q++) atomicAdd(&sb[q * nbin + cur], acc[q]);
        for (int q = 0; q < PK_Q; q++) acc[q] = 0.f;
        cur = b;
      }
      acc[0] += 1.0f;                                      // number of modes
      acc[1] += kr;                                        // k
      acc[2] += (a.x * a.x + a.y * a.y) * w;               // auto power 1
      acc[3] += (bb.x * bb.x + bb.y * bb.y) * w;           // auto power 2
      acc[4] += (a.x * bb.x + a.y * bb.y) * w;             // cross power
      acc[5] += 1.0f / s2;                                 // kernel 1
      acc[6] += 1.0f / s4;                                 // kernel 2
    }
    if (cur >= 0 && cur < nbin)
      for (int q = 0; q < PK_Q; q++) atomicAdd(&sb[q * nbin + cur], acc[q]);
  }
  __syncthreads();
  float* out = part + (int64_t)blockIdx.x * PK_Q * nbin;
  for (int i = threadIdx.x; i < PK_Q * nbin; i += blockDim.x) out[i] = sb[i];
}

// sum of the per-block partial bins in FP64
__global__ void k_pk_reduce(const float* __restrict__ part, int nblocks, int n, double* __restrict__ out) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int b = 0; b < nblocks; b++) s += (double)part[(int64_t)b * n + i];
    out[i] = s;
  }
}

}  // namespace

// nbin=nint(nyquest*sqrt(3.)) in real(4) (powerspectrum.f90:11)
extern "C" int cube_pk_nbin(int ng) { return (int)std::lround((double)((float)(ng / 2) * std::sqrt(3.0f))); }

extern "C" int cube_power_spectrum(cube_ctx* c, int ng, float box, const float* delta2, double* xi, int nbin) {
  if (!c || !xi) return CUBE_ERR_ARG;
  if (!c->have_state) return cube_fail(c, CUBE_ERR_STATE, "no state uploaded");
  if (ng != c->p.nc && ng != 2 * c->p.nc && ng != 4 * c->p.nc)
    return cube_fail(c, CUBE_ERR_ARG, "power-spectrum mesh must be nc, 2nc or 4nc per dimension");
  if (ng % 2) return cube_fail(c, CUBE_ERR_ARG, "power-spectrum mesh must be even");
  const int need = cube_pk_nbin(ng);
  if (nbin < need) return cube_fail(c, CUBE_ERR_ARG, "xi needs nint(ng/2*sqrt(3)) bins");
  CUBE_CUDA(c, cudaSetDevice(c->device));
  if (int r = cube_upload_join(c)) return r;
  cudaStream_t s = c->stream;
  float* m1 = c->force_f[0];
  float* m2 = c->force_f[1];
  float* part = c->force_f[2];
  // 1. CIC density, mass 1, and its exact total
  CUBE_CUDA(c, cudaMemsetAsync(m1, 0, sizeof(float) * (size_t)(ng + 2) * ng * ng, s));
  CUBE_CUDA(c, cudaMemsetAsync(&c->dstats->rhof_fix, 0, 8, s));
  int r = cube_pk_deposit(c, ng, m1, &c->dstats->rhof_fix);
  if (r) return r;
  r = cube_stats_fetch(c);
  if (r) return r;
  const double total = std::ldexp((double)c->hstats->rhof_fix, -dep_shift(1.0f));
  if (!(total > 0.0)) return cube_fail(c, CUBE_ERR_STATE, "no mass on the mesh");
  const double mean = total / ((double)ng * ng * ng);
  k_pk_delta<<<cube_grid((int64_t)ng * ng, 1, 8), 256, 0, s>>>(m1, ng, (float)(1.0 / mean));
  CUBE_CUDA(c, cudaGetLastError());
  // 2. transforms: the fine or coarse plan when the mesh matches, else one made here
  cufftHandle plan = 0;
  bool own = false;
  if (ng == c->nf) {
    plan = c->plan_f_r2c;
  } else if (ng == c->p.nc) {
    plan = c->plan_c_r2c;
  } else {
    CUBE_FFT(c, cufftPlan3d(&plan, ng, ng, ng, CUFFT_R2C));
    CUBE_FFT(c, cufftSetStream(plan, s));
    own = true;
  }
  cufftResult fr = cufftExecR2C(plan, m1, (cufftComplex*)m1);
  if (fr == CUFFT_SUCCESS && delta2) {
    cudaError_t e = cudaMemcpy2DAsync(m2, sizeof(float) * (ng + 2), delta2, sizeof(float) * ng, sizeof(float) * ng,
                                      (size_t)ng * ng, cudaMemcpyHostToDevice, s);
    fr = e == cudaSuccess ? cufftExecR2C(plan, m2, (cufftComplex*)m2) : CUFFT_EXEC_FAILED;
  }
  if (own) cufftDestroy(plan);
  if (fr != CUFFT_SUCCESS) return cube_fail(c, CUBE_ERR_CUDA, "power-spectrum FFT failed");
  // 3. binned sums
  const int nb = cube_grid((int64_t)ng * ng, PK_T, 4);
  const size_t smem = sizeof(float) * PK_Q * need;
  CUBE_CUDA(c, cudaFuncSetAttribute(k_pk_bin, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  k_pk_bin<<<nb, PK_T, smem, s>>>((const float2*)m1, (const float2*)(delta2 ? m2 : m1), ng, need, part);
  CUBE_CUDA(c, cudaGetLastError());
  double* sums = reinterpret_cast<double*>(part + (((size_t)nb * PK_Q * need + 64) & ~(size_t)63));
  k_pk_reduce<<<cube_grid(PK_Q * need, 256), 256, 0, s>>>(part, nb, PK_Q * need, sums);
  CUBE_CUDA(c, cudaGetLastError());
  std::vector<double> h((size_t)PK_Q * need);
  CUBE_CUDA(c, cudaMemcpyAsync(h.data(), sums, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, s));
  CUBE_CUDA(c, cudaStreamSynchronize(s));
  // 4. normalisation (powerspectrum.f90:121-133); empty bins divide by zero
  //    as in the reference
  const double two_pi = 2.0 * (double)CUBE_PI_F;
  for (int b = 0; b < nbin; b++) {
    double* o = xi + 10 * (size_t)b;
    if (b >= need) {
      for (int q = 0; q < 10; q++) o[q] = 0.0;
      continue;
    }
    double v[PK_Q];
    for (int q = 0; q < PK_Q; q++) v[q] = h[(size_t)q * need + b];
    o[0] = v[0];
    o[1] = v[1] / v[0] * two_pi / (double)box;
    for (int q = 2; q < PK_Q; q++) o[q] = v[q] / v[0];
    o[7] = o[4] / std::sqrt(o[2] * o[3]);
    o[8] = std::sqrt(o[3] / o[2]);
    o[9] = std::pow(o[7], 4) / (o[8] * o[8]) * o[3];
  }
  return CUBE_OK;
}
