// cube_dpm.cu -- the differentiable form of the PM step: a single-level
// particle-mesh integrator on decoded FP32 positions with hand-written adjoint
// kernels, for gradients of a loss of the final state with respect to the
// initial white noise.
//
// Forward map (all FP32; the state is each particle's displacement d from its
// lattice point q = step*l + 0.5, in mesh cells, and its velocity v):
//   IC      noise (npd^3 lattice) -> phi = C2R(filter * R2C(noise)), the
//           initial-condition filter of cube_ic.cu (Delta^2 scaling times the
//           corrected discrete potential kernel, initial_conditions.f90:306-330,
//           433-541) on the particle lattice; Zel'dovich displacement and
//           velocity from central differences of phi (:702-769):
//             d = -step*gd/(8 pi),  v = -step*gd*a^2H/(8 pi)
//   step i  drift  d += drift_i * v              (update_particle.f90:66, dt_mid)
//           CIC deposit of mass m on the cell-centred periodic ng^3 mesh
//           phi = C2R(G * R2C(rho)), G = -4 pi / khat^2 (khat = 2 sin(pi k/ng))
//           F = -(phi(c+e) - phi(c-e))/2, CIC-interpolated to the particle
//           kick   v += kick_i * F                (pm.f90:162, a_mid*dt/6/pi)
// Adjoint kernels (one per forward kernel):
//   kick    -> k_dpm_kick_adj: the interpolation-scatter of kick*vbar through
//              the central differences onto the potential's 32-point stencil
//              (one FP32 reduction per point), plus the direct term of the
//              moving weights (grad w . F)
//   Green   -> the same multiply: C2R o G o R2C is symmetric for a real even G
//   deposit -> k_dpm_deposit_adj: the transpose-gather m * grad w . rhobar,
//              then the drift's transpose vbar += drift_i * xbar
//   IC      -> k_dpm_ic_adj (the transpose of the central differences, a
//              gather per lattice point) and the symmetric filter again.
// Positions are never formed as FP32 absolutes: the CIC cell is the lattice
// point's integer cell plus floor(d), the weights come from d - floor(d), so
// the weights keep FP32 precision of d (a few cells) instead of that of a
// coordinate up to ng -- the same reason CUBE stores in-cell offsets.
// Memory is bounded by step checkpointing: the state (x, v) is kept at the
// start of every segment of ckpt_every steps; the backward pass re-runs each
// segment forward, keeping its post-drift positions and potentials, and then
// walks it in reverse.  The forward and backward passes are
// each one captured CUDA graph (rebuilt when the schedule changes).  Both
// scatters -- the CIC deposit and the adjoint's stencil scatter -- sum in
// 64-bit fixed point (integer atomics, exact and order-independent) and are
// converted to FP32 once, so every pass gives the same bits run to run.  The
// deposit's scale follows from the mass and particle count; the stencil
// scatter's from the largest velocity cotangent, reduced on the device first.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "cube_internal.cuh"

namespace {
// lattice of the particles: npd points per dimension, step mesh cells apart
struct Lattice {
  int npd, step, ng;
  FastDiv dnpd;
};
}  // namespace

struct cube_dpm {
  cube_ctx base;  // device, stream and error text
  Lattice lat_{};
  cube_dpm_params p{};
  int ng = 0, npd = 0, step = 0;
  int64_t np = 0;
  float mass = 0.f, vf = 0.f;
  cufftHandle pm_r2c = 0, pm_c2r = 0, ic_r2c = 0, ic_c2r = 0;
  float* green = nullptr;  // (ng/2+1) ng^2, 1/ng^3 folded in
  float* filt = nullptr;   // (npd/2+1) npd^2, 1/npd^3 folded in
  float* mesh = nullptr;   // padded ng^3: rho / phi
  float* adj = nullptr;    // padded ng^3: phibar / rhobar
  long long* fix = nullptr;  // ng^3 fixed-point sums of the scatters (zero between uses)
  unsigned int* gmax = nullptr;  // device: max |gv| (float bits) for the stencil scatter's scale
  int dep_shift = 0;       // the deposit's fixed point: value = integer * 2^-dep_shift
  float* lat = nullptr;    // padded npd^3: noise / IC potential / their adjoints
  float *x = nullptr, *v = nullptr, *gx = nullptr, *gv = nullptr;
  float* seg = nullptr;    // segment starts: nseg x (x, v)
  float* pos = nullptr;    // post-drift positions of one segment
  float* phis = nullptr;   // potentials of one segment: ckpt_every padded meshes
  std::vector<float> drift, kick;
  int nsteps = 0;
  cudaGraphExec_t gfwd = nullptr, gbwd = nullptr;
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
  float fwd_ms = 0.f, bwd_ms = 0.f;
  int64_t nforward = 0;  // forward passes run; the backward needs one
};

namespace {

constexpr float kInv8Pi = (float)(1.0 / (8.0 * 3.14159265358979323846));

__device__ __forceinline__ int64_t pad_at(int n, int x, int y, int z) {
  return x + (int64_t)(n + 2) * (y + (int64_t)n * z);
}

// CIC stencil of one particle on the cell-centred periodic mesh: wrapped
// coordinates of the offsets -1..2 around the cell of x - 0.5 = step*l + d
// per axis, and the weights of offsets 0 and 1.
struct Cic {
  int i[3][4];
  float w[3][2];
};
__device__ __forceinline__ void cic_setup(int64_t p, const float* dp, const Lattice& L, Cic& c) {
  const uint32_t q1 = fdiv((uint32_t)p, L.dnpd), q2 = fdiv(q1, L.dnpd);
  const int li[3] = {(int)((uint32_t)p - q1 * (uint32_t)L.npd), (int)(q1 - q2 * (uint32_t)L.npd), (int)q2};
  const int ng = L.ng;
#pragma unroll
  for (int e = 0; e < 3; e++) {
    const float fl = floorf(dp[e]);
    const float f = dp[e] - fl;
    int b = wrapi(L.step * li[e] + (int)fmaxf(fminf(fl, 1.0e6f), -1.0e6f) - 1, ng);
#pragma unroll
    for (int t = 0; t < 4; t++) {
      c.i[e][t] = b;
      b = b + 1 == ng ? 0 : b + 1;
    }
    c.w[e][0] = 1.0f - f;
    c.w[e][1] = f;
  }
}

// The 32 potential values the interpolated central-difference force reads:
// the 2x2x2 core and, per axis, the faces at offsets -1 (lo) and 2 (hi).
// core[z][y][x]; lo/hi[0][z][y], lo/hi[1][z][x], lo/hi[2][y][x].
struct Stencil {
  float core[2][2][2];
  float lo[3][2][2], hi[3][2][2];
};
__device__ __forceinline__ void stencil_load(const float* __restrict__ m, int ng, const Cic& c, Stencil& s) {
#pragma unroll
  for (int a = 0; a < 2; a++)
#pragma unroll
    for (int b = 0; b < 2; b++) {
#pragma unroll
      for (int x = 0; x < 2; x++) s.core[a][b][x] = __ldg(m + pad_at(ng, c.i[0][1 + x], c.i[1][1 + b], c.i[2][1 + a]));
      s.lo[0][a][b] = __ldg(m + pad_at(ng, c.i[0][0], c.i[1][1 + b], c.i[2][1 + a]));
      s.hi[0][a][b] = __ldg(m + pad_at(ng, c.i[0][3], c.i[1][1 + b], c.i[2][1 + a]));
      s.lo[1][a][b] = __ldg(m + pad_at(ng, c.i[0][1 + b], c.i[1][0], c.i[2][1 + a]));
      s.hi[1][a][b] = __ldg(m + pad_at(ng, c.i[0][1 + b], c.i[1][3], c.i[2][1 + a]));
      s.lo[2][a][b] = __ldg(m + pad_at(ng, c.i[0][1 + b], c.i[1][1 + a], c.i[2][0]));
      s.hi[2][a][b] = __ldg(m + pad_at(ng, c.i[0][1 + b], c.i[1][1 + a], c.i[2][3]));
    }
}
// dense index of the fixed-point sums
__device__ __forceinline__ int64_t dense_at(int n, int x, int y, int z) { return x + (int64_t)n * (y + (int64_t)n * z); }
// add v * 2^sh, rounded to an integer, to a fixed-point sum (two's complement
// in an unsigned 64-bit atomic: the total is exact and independent of order)
__device__ __forceinline__ void fix_add(long long* m, int64_t i, float v, float scale) {
  atomicAdd(reinterpret_cast<unsigned long long*>(m) + i, (unsigned long long)__float2ll_rn(v * scale));
}
__device__ __forceinline__ void stencil_add(long long* __restrict__ m, int ng, const Cic& c, const Stencil& s,
                                            float scale) {
#pragma unroll
  for (int a = 0; a < 2; a++)
#pragma unroll
    for (int b = 0; b < 2; b++) {
#pragma unroll
      for (int x = 0; x < 2; x++) fix_add(m, dense_at(ng, c.i[0][1 + x], c.i[1][1 + b], c.i[2][1 + a]), s.core[a][b][x], scale);
      fix_add(m, dense_at(ng, c.i[0][0], c.i[1][1 + b], c.i[2][1 + a]), s.lo[0][a][b], scale);
      fix_add(m, dense_at(ng, c.i[0][3], c.i[1][1 + b], c.i[2][1 + a]), s.hi[0][a][b], scale);
      fix_add(m, dense_at(ng, c.i[0][1 + b], c.i[1][0], c.i[2][1 + a]), s.lo[1][a][b], scale);
      fix_add(m, dense_at(ng, c.i[0][1 + b], c.i[1][3], c.i[2][1 + a]), s.hi[1][a][b], scale);
      fix_add(m, dense_at(ng, c.i[0][1 + b], c.i[1][1 + a], c.i[2][0]), s.lo[2][a][b], scale);
      fix_add(m, dense_at(ng, c.i[0][1 + b], c.i[1][1 + a], c.i[2][3]), s.hi[2][a][b], scale);
    }
}

// The stencil scatter's fixed point: every value it adds is at most
// 0.5*|kick|*max|gv| and a mesh point receives at most 32 of them from each of
// np particles, so sums stay below 2^61 with scale 2^sh, sh = 60 - ilogb(16 *
// |kick| * np * max|gv|).  Derived on the device from the reduced maximum.
__device__ __forceinline__ int adj_shift(float kick, int64_t np, const unsigned int* gmax) {
  const float g = __uint_as_float(*gmax);
  if (!(g > 0.f)) return 0;
  const double bound = 16.0 * (double)fabsf(kick) * (double)np * (double)g;
  return 60 - ilogb(bound);
}
// 2^sh as a float (sh within the float exponent range)
__device__ __forceinline__ float pow2f(int sh) { return ldexpf(1.0f, max(-126, min(127, sh))); }

// max |gv| over the particles (float bits, non-negative: integer max orders them)
__global__ void k_dpm_absmax(const float* __restrict__ v, int64_t n, unsigned int* __restrict__ out) {
  float m = 0.f;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    m = fmaxf(m, fabsf(v[i]));
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax(out, __float_as_uint(m));
}

// fixed-point sums -> the padded FP32 mesh, zeroing the sums for their next use;
// sh = the scatter's shift (from the host, or from adj_shift when gmax is set)
__global__ void k_dpm_fix_out(long long* __restrict__ fix, int ng, int sh, float kick, int64_t np,
                              const unsigned int* __restrict__ gmax, float* __restrict__ mesh) {
  if (gmax) sh = adj_shift(kick, np, gmax);
  const int64_t n = (int64_t)ng * ng * ng;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const long long q = fix[i];
    fix[i] = 0;
    const int x = (int)(i % ng);
    const int64_t yz = i / ng;
    // integer -> nearest float, then the exact power-of-two scale
    mesh[x + (int64_t)(ng + 2) * yz] = ldexpf(__ll2float_rn(q), -sh);
  }
}

// the central-difference force component d at corner (ax, ay, az) is
// 0.5*(minus - plus); references to the two stencil values it reads
__device__ __forceinline__ float& plus_ref(Stencil& s, int d, int ax, int ay, int az) {
  if (d == 0) return ax == 0 ? s.core[az][ay][1] : s.hi[0][az][ay];
  if (d == 1) return ay == 0 ? s.core[az][1][ax] : s.hi[1][az][ax];
  return az == 0 ? s.core[1][ay][ax] : s.hi[2][ay][ax];
}
__device__ __forceinline__ float& minus_ref(Stencil& s, int d, int ax, int ay, int az) {
  if (d == 0) return ax == 0 ? s.lo[0][az][ay] : s.core[az][ay][0];
  if (d == 1) return ay == 0 ? s.lo[1][az][ax] : s.core[az][0][ax];
  return az == 0 ? s.lo[2][ay][ax] : s.core[0][ay][ax];
}

// ------------------------------------------------------------------ kernels
// d' = d + drift*v (when v is given), stored to dout / pos when given, then
// the CIC deposit of mass at d'
// (dout may be din: each thread reads its particle before writing it)
__global__ void __launch_bounds__(256) k_dpm_deposit(const float* xin, const float* __restrict__ vin, float drift,
                                                     int64_t np, Lattice L, float mass, float* xout,
                                                     float* __restrict__ pos, long long* __restrict__ fix,
                                                     float scale) {
  const int ng = L.ng;
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < np; p += (int64_t)gridDim.x * blockDim.x) {
    float x[3];
#pragma unroll
    for (int e = 0; e < 3; e++) {
      x[e] = xin[3 * p + e];
      if (vin) x[e] = x[e] + drift * vin[3 * p + e];
    }
#pragma unroll
    for (int e = 0; e < 3; e++) {
      if (xout) xout[3 * p + e] = x[e];
      if (pos) pos[3 * p + e] = x[e];
    }
    Cic c;
    cic_setup(p, x, L, c);
#pragma unroll
    for (int az = 0; az < 2; az++)
#pragma unroll
      for (int ay = 0; ay < 2; ay++)
#pragma unroll
        for (int ax = 0; ax < 2; ax++)
          fix_add(fix, dense_at(ng, c.i[0][1 + ax], c.i[1][1 + ay], c.i[2][1 + az]),
                  mass * (c.w[0][ax] * c.w[1][ay] * c.w[2][az]), scale);
  }
}

// spectrum *= g (real), one complex value per entry
__global__ void k_dpm_mul(float2* __restrict__ s, const float* __restrict__ g, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float2 a = s[i];
    const float f = g[i];
    s[i] = make_float2(a.x * f, a.y * f);
  }
}

// G = -4 pi / khat^2 / ng^3 on the half spectrum, 0 at k = 0
__global__ void k_dpm_green(float* __restrict__ g, int ng) {
  const int nh = ng / 2 + 1;
  const int64_t n = (int64_t)nh * ng * ng;
  const float inv = 1.0f / ((float)ng * (float)ng * (float)ng);
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int x = (int)(i % nh), y = (int)((i / nh) % ng), z = (int)(i / ((int64_t)nh * ng));
    const float sx = 2.0f * sinpif((float)x / (float)ng), sy = 2.0f * sinpif((float)y / (float)ng),
                sz = 2.0f * sinpif((float)z / (float)ng);
    const float k2 = sx * sx + sy * sy + sz * sz;
    g[i] = i == 0 ? 0.f : -4.0f * CUBE_PI_F / k2 * inv;
  }
}

// v += kick * F(x), F the CIC-interpolated central-difference force of phi
__global__ void __launch_bounds__(256) k_dpm_kick(const float* __restrict__ x, float* __restrict__ v, int64_t np,
                                                  Lattice L, const float* __restrict__ phi, float kick) {
  const int ng = L.ng;
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < np; p += (int64_t)gridDim.x * blockDim.x) {
    const float xp[3] = {x[3 * p], x[3 * p + 1], x[3 * p + 2]};
    Cic c;
    cic_setup(p, xp, L, c);
    Stencil s;
    stencil_load(phi, ng, c, s);
    float f[3] = {0.f, 0.f, 0.f};
#pragma unroll
    for (int az = 0; az < 2; az++)
#pragma unroll
      for (int ay = 0; ay < 2; ay++)
#pragma unroll
        for (int ax = 0; ax < 2; ax++) {
          const float w = c.w[0][ax] * c.w[1][ay] * c.w[2][az];
#pragma unroll
          for (int d = 0; d < 3; d++)
            f[d] += w * (0.5f * (minus_ref(s, d, ax, ay, az) - plus_ref(s, d, ax, ay, az)));
        }
#pragma unroll
    for (int d = 0; d < 3; d++) v[3 * p + d] += kick * f[d];
  }
}

// adjoint of the kick at positions x with velocity cotangent gv (unchanged by
// the kick): gx += kick * sum_d gv_d * grad(w) . F_d (the weights move with x),
// and phibar += the interpolation-scatter of kick * gv through the central
// differences
__global__ void __launch_bounds__(256) k_dpm_kick_adj(const float* __restrict__ x, const float* __restrict__ gv,
                                                      int64_t np, Lattice L, const float* __restrict__ phi, float kick,
                                                      float* __restrict__ gx, long long* __restrict__ phibar,
                                                      const unsigned int* __restrict__ gmax) {
  const int ng = L.ng;
  const float scale = pow2f(adj_shift(kick, np, gmax));
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < np; p += (int64_t)gridDim.x * blockDim.x) {
    const float xp[3] = {x[3 * p], x[3 * p + 1], x[3 * p + 2]};
    const float g[3] = {kick * gv[3 * p], kick * gv[3 * p + 1], kick * gv[3 * p + 2]};
    Cic c;
    cic_setup(p, xp, L, c);
    Stencil s;
    stencil_load(phi, ng, c, s);
    Stencil b;
#pragma unroll
    for (int a = 0; a < 2; a++)
#pragma unroll
      for (int q = 0; q < 2; q++) {
#pragma unroll
        for (int t = 0; t < 2; t++) b.core[a][q][t] = 0.f;
#pragma unroll
        for (int d = 0; d < 3; d++) b.lo[d][a][q] = b.hi[d][a][q] = 0.f;
      }
    float gxp[3] = {0.f, 0.f, 0.f};
#pragma unroll
    for (int az = 0; az < 2; az++)
#pragma unroll
      for (int ay = 0; ay < 2; ay++)
#pragma unroll
        for (int ax = 0; ax < 2; ax++) {
          const float wx = c.w[0][ax], wy = c.w[1][ay], wz = c.w[2][az];
          const float w = wx * wy * wz;
          float gf = 0.f;  // sum_d g_d F_d at this corner
#pragma unroll
          for (int d = 0; d < 3; d++) {
            gf += g[d] * (0.5f * (minus_ref(s, d, ax, ay, az) - plus_ref(s, d, ax, ay, az)));
            const float h = 0.5f * w * g[d];
            minus_ref(b, d, ax, ay, az) += h;
            plus_ref(b, d, ax, ay, az) -= h;
          }
          // d w / d x_e = (a_e ? 1 : -1) * product of the other two weights
          gxp[0] += (ax ? gf : -gf) * (wy * wz);
          gxp[1] += (ay ? gf : -gf) * (wx * wz);
          gxp[2] += (az ? gf : -gf) * (wx * wy);
        }
#pragma unroll
    for (int e = 0; e < 3; e++) gx[3 * p + e] += gxp[e];
    stencil_add(phibar, ng, c, b, scale);
  }
}

// adjoint of the deposit at positions x: gx += mass * grad(w) . rhobar; then
// the drift's transpose gv += drift * gx (gv may be null)
__global__ void __launch_bounds__(256) k_dpm_deposit_adj(const float* __restrict__ x, int64_t np, Lattice L,
                                                         const float* __restrict__ rhobar, float mass, float drift,
                                                         float* __restrict__ gx, float* __restrict__ gv,
                                                         int accumulate) {
  const int ng = L.ng;
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < np; p += (int64_t)gridDim.x * blockDim.x) {
    const float xp[3] = {x[3 * p], x[3 * p + 1], x[3 * p + 2]};
    Cic c;
    cic_setup(p, xp, L, c);
    float gxp[3] = {0.f, 0.f, 0.f};
#pragma unroll
    for (int az = 0; az < 2; az++)
#pragma unroll
      for (int ay = 0; ay < 2; ay++)
#pragma unroll
        for (int ax = 0; ax < 2; ax++) {
          const float r = __ldg(rhobar + pad_at(ng, c.i[0][1 + ax], c.i[1][1 + ay], c.i[2][1 + az]));
          const float wx = c.w[0][ax], wy = c.w[1][ay], wz = c.w[2][az];
          gxp[0] += (ax ? r : -r) * (wy * wz);
          gxp[1] += (ay ? r : -r) * (wx * wz);
          gxp[2] += (az ? r : -r) * (wx * wy);
        }
#pragma unroll
    for (int e = 0; e < 3; e++) {
      const float t = (accumulate ? gx[3 * p + e] : 0.f) + mass * gxp[e];
      gx[3 * p + e] = t;
      if (gv) gv[3 * p + e] += drift * t;
    }
  }
}

// Zel'dovich state from the lattice potential phi (padded npd^3, normalised):
// particle l's lattice point is mesh cell step*l; gd = phi(l+e) - phi(l-e)
__global__ void k_dpm_ic(const float* __restrict__ phi, int npd, int step, float vf, float* __restrict__ x,
                         float* __restrict__ v) {
  const int64_t n = (int64_t)npd * npd * npd;
  for (int64_t l = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; l < n; l += (int64_t)gridDim.x * blockDim.x) {
    const int li[3] = {(int)(l % npd), (int)((l / npd) % npd), (int)(l / ((int64_t)npd * npd))};
#pragma unroll
    for (int d = 0; d < 3; d++) {
      int up[3] = {li[0], li[1], li[2]}, dn[3] = {li[0], li[1], li[2]};
      up[d] = up[d] + 1 == npd ? 0 : up[d] + 1;
      dn[d] = dn[d] == 0 ? npd - 1 : dn[d] - 1;
      const float gd = phi[pad_at(npd, up[0], up[1], up[2])] - phi[pad_at(npd, dn[0], dn[1], dn[2])];
      const float s = (float)step * gd * kInv8Pi;
      x[3 * l + d] = -s;
      v[3 * l + d] = -s * vf;
    }
  }
}

// transpose of k_dpm_ic: phibar(m) = sum_d gbar_d(m - e_d) - gbar_d(m + e_d),
// gbar_d(p) = -step/(8 pi) * (gx_d(p) + vf * gv_d(p)); one thread per lattice point
__global__ void k_dpm_ic_adj(const float* __restrict__ gx, const float* __restrict__ gv, int npd, int step, float vf,
                             float* __restrict__ phibar) {
  const int64_t n = (int64_t)npd * npd * npd;
  const float cst = -(float)step * kInv8Pi;
  for (int64_t m = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; m < n; m += (int64_t)gridDim.x * blockDim.x) {
    const int li[3] = {(int)(m % npd), (int)((m / npd) % npd), (int)(m / ((int64_t)npd * npd))};
    float acc = 0.f;
#pragma unroll
    for (int d = 0; d < 3; d++) {
      int up[3] = {li[0], li[1], li[2]}, dn[3] = {li[0], li[1], li[2]};
      up[d] = up[d] + 1 == npd ? 0 : up[d] + 1;
      dn[d] = dn[d] == 0 ? npd - 1 : dn[d] - 1;
      const int64_t pu = up[0] + (int64_t)npd * (up[1] + (int64_t)npd * up[2]);
      const int64_t pd = dn[0] + (int64_t)npd * (dn[1] + (int64_t)npd * dn[2]);
      const float gu = cst * (gx[3 * pu + d] + vf * gv[3 * pu + d]);
      const float gdn = cst * (gx[3 * pd + d] + vf * gv[3 * pd + d]);
      acc += gdn - gu;
    }
    phibar[pad_at(npd, li[0], li[1], li[2])] = acc;
  }
}

// ------------------------------------------------------------------ host
int dpm_fail(cube_dpm* d, int code, const std::string& m) { return cube_fail(&d->base, code, m); }

size_t pad_bytes(int n) { return sizeof(float) * (size_t)(n + 2) * n * n; }
size_t spec_count(int n) { return (size_t)(n / 2 + 1) * n * n; }

int make_plan(cube_dpm* d, cufftHandle* h, int n, cufftType t) {
  cube_ctx* c = &d->base;
  CUBE_FFT(c, cufftPlan3d(h, n, n, n, t));
  CUBE_FFT(c, cufftSetStream(*h, c->stream));
  return CUBE_OK;
}

// phi = C2R(g * R2C(m)) in place on a padded n^3 mesh
int spectral(cube_dpm* d, float* m, const float* g, int n, cufftHandle r2c, cufftHandle c2r) {
  cube_ctx* c = &d->base;
  CUBE_FFT(c, cufftExecR2C(r2c, m, (cufftComplex*)m));
  const int64_t ns = (int64_t)spec_count(n);
  k_dpm_mul<<<cube_grid(ns, 256), 256, 0, c->stream>>>((float2*)m, g, ns);
  CUBE_CUDA(c, cudaGetLastError());
  CUBE_FFT(c, cufftExecC2R(c2r, (cufftComplex*)m, m));
  return CUBE_OK;
}

// fixed-point sums (zero on entry, zero again on return) -> the padded mesh
int fix_out(cube_dpm* d, float* mesh, int sh, float kick = 0.f, const unsigned int* gmax = nullptr) {
  cube_ctx* c = &d->base;
  const int64_t n = (int64_t)d->ng * d->ng * d->ng;
  k_dpm_fix_out<<<cube_grid(n, 256), 256, 0, c->stream>>>(d->fix, d->ng, sh, kick, d->np, gmax, mesh);
  CUBE_CUDA(c, cudaGetLastError());
  return CUBE_OK;
}

int deposit(cube_dpm* d, const float* xin, const float* vin, float drift, float* xout, float* pos,
            float* mesh = nullptr) {
  cube_ctx* c = &d->base;
  if (!mesh) mesh = d->mesh;
  k_dpm_deposit<<<cube_grid(d->np, 256), 256, 0, c->stream>>>(xin, vin, drift, d->np, d->lat_, d->mass, xout, pos,
                                                               d->fix, std::ldexp(1.0f, d->dep_shift));
  CUBE_CUDA(c, cudaGetLastError());
  return fix_out(d, mesh, d->dep_shift);
}

int nseg(const cube_dpm* d) { return (d->nsteps + d->p.ckpt_every - 1) / d->p.ckpt_every; }

// the forward pass: IC from the noise in lat, then every step; (x, v) at each
// segment start into seg
int record_forward(cube_dpm* d) {
  cube_ctx* c = &d->base;
  cudaStream_t s = c->stream;
  const size_t sb = sizeof(float) * 3 * (size_t)d->np;
  int r = spectral(d, d->lat, d->filt, d->npd, d->ic_r2c, d->ic_c2r);
  if (r) return r;
  k_dpm_ic<<<cube_grid(d->np, 256), 256, 0, s>>>(d->lat, d->npd, d->step, d->vf, d->x, d->v);
  CUBE_CUDA(c, cudaGetLastError());
  for (int i = 0; i < d->nsteps; i++) {
    if (i % d->p.ckpt_every == 0) {
      float* slot = d->seg + (size_t)(i / d->p.ckpt_every) * 6 * d->np;
      CUBE_CUDA(c, cudaMemcpyAsync(slot, d->x, sb, cudaMemcpyDeviceToDevice, s));
      CUBE_CUDA(c, cudaMemcpyAsync(slot + 3 * d->np, d->v, sb, cudaMemcpyDeviceToDevice, s));
    }
    if ((r = deposit(d, d->x, d->v, d->drift[i], d->x, nullptr))) return r;
    if ((r = spectral(d, d->mesh, d->green, d->ng, d->pm_r2c, d->pm_c2r))) return r;
    k_dpm_kick<<<cube_grid(d->np, 256), 256, 0, s>>>(d->x, d->v, d->np, d->lat_, d->mesh, d->kick[i]);
    CUBE_CUDA(c, cudaGetLastError());
  }
  return CUBE_OK;
}

// the backward pass from the cotangents (gx, gv) of the final state to those
// of the initial state (left in gx, gv) and of the noise (left in lat)
int record_backward(cube_dpm* d) {
  cube_ctx* c = &d->base;
  cudaStream_t s = c->stream;
  const size_t sb = sizeof(float) * 3 * (size_t)d->np;
  const int64_t np = d->np;
  int r;
  for (int j = nseg(d) - 1; j >= 0; j--) {
    const int i0 = j * d->p.ckpt_every;
    const int i1 = std::min(i0 + d->p.ckpt_every, d->nsteps);
    const float* slot = d->seg + (size_t)j * 6 * np;
    CUBE_CUDA(c, cudaMemcpyAsync(d->x, slot, sb, cudaMemcpyDeviceToDevice, s));
    CUBE_CUDA(c, cudaMemcpyAsync(d->v, slot + 3 * np, sb, cudaMemcpyDeviceToDevice, s));
    // re-run the segment, keeping the post-drift positions and potentials
    for (int i = i0; i < i1; i++) {
      float* pos = d->pos + (size_t)(i - i0) * 3 * np;
      float* phi = d->phis + (size_t)(i - i0) * (pad_bytes(d->ng) / sizeof(float));
      if ((r = deposit(d, d->x, d->v, d->drift[i], d->x, pos, phi))) return r;
      if ((r = spectral(d, phi, d->green, d->ng, d->pm_r2c, d->pm_c2r))) return r;
      if (i + 1 < i1) {
        k_dpm_kick<<<cube_grid(np, 256), 256, 0, s>>>(d->x, d->v, np, d->lat_, phi, d->kick[i]);
        CUBE_CUDA(c, cudaGetLastError());
      }
    }
    // walk it in reverse
    for (int i = i1 - 1; i >= i0; i--) {
      const float* pos = d->pos + (size_t)(i - i0) * 3 * np;
      const float* phi = d->phis + (size_t)(i - i0) * (pad_bytes(d->ng) / sizeof(float));
      CUBE_CUDA(c, cudaMemsetAsync(d->gmax, 0, sizeof(unsigned int), s));
      k_dpm_absmax<<<cube_grid(3 * np, 256, 4), 256, 0, s>>>(d->gv, 3 * np, d->gmax);
      k_dpm_kick_adj<<<cube_grid(np, 256), 256, 0, s>>>(pos, d->gv, np, d->lat_, phi, d->kick[i], d->gx, d->fix,
                                                         d->gmax);
      CUBE_CUDA(c, cudaGetLastError());
      if ((r = fix_out(d, d->adj, 0, d->kick[i], d->gmax))) return r;
      if ((r = spectral(d, d->adj, d->green, d->ng, d->pm_r2c, d->pm_c2r))) return r;
      k_dpm_deposit_adj<<<cube_grid(np, 256), 256, 0, s>>>(pos, np, d->lat_, d->adj, d->mass, d->drift[i], d->gx, d->gv,
                                                            1);
      CUBE_CUDA(c, cudaGetLastError());
    }
  }
  // the initial conditions
  k_dpm_ic_adj<<<cube_grid(np, 256), 256, 0, s>>>(d->gx, d->gv, d->npd, d->step, d->vf, d->lat);
  CUBE_CUDA(c, cudaGetLastError());
  return spectral(d, d->lat, d->filt, d->npd, d->ic_r2c, d->ic_c2r);
}

int capture(cube_dpm* d, int (*rec)(cube_dpm*), cudaGraphExec_t* out) {
  cube_ctx* c = &d->base;
  cudaGraph_t g = nullptr;
  CUBE_CUDA(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
  int r = rec(d);
  cudaError_t e = cudaStreamEndCapture(c->stream, &g);
  if (r) {
    if (g) cudaGraphDestroy(g);
    return r;
  }
  if (e != cudaSuccess) return dpm_fail(d, CUBE_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
  e = cudaGraphInstantiate(out, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return dpm_fail(d, CUBE_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
  return CUBE_OK;
}

void drop_graphs(cube_dpm* d) {
  if (d->gfwd) cudaGraphExecDestroy(d->gfwd);
  if (d->gbwd) cudaGraphExecDestroy(d->gbwd);
  d->gfwd = d->gbwd = nullptr;
}

void release(cube_dpm* d) {
  cudaSetDevice(d->base.device);
  drop_graphs(d);
  for (cudaEvent_t e : d->ev)
    if (e) cudaEventDestroy(e);
  for (cufftHandle h : {d->pm_r2c, d->pm_c2r, d->ic_r2c, d->ic_c2r})
    if (h) cufftDestroy(h);
  for (void* b : {(void*)d->green, (void*)d->filt, (void*)d->mesh, (void*)d->adj, (void*)d->lat, (void*)d->x,
                  (void*)d->v, (void*)d->gx, (void*)d->gv, (void*)d->seg, (void*)d->pos, (void*)d->phis,
                  (void*)d->fix, (void*)d->gmax})
    if (b) cudaFree(b);
  if (d->base.stream) cudaStreamDestroy(d->base.stream);
  d->base.stream = nullptr;
}

int dalloc(cube_dpm* d, float** p, size_t bytes) {
  cudaError_t e = cudaMalloc((void**)p, bytes ? bytes : 16);
  if (e != cudaSuccess)
    return dpm_fail(d, CUBE_ERR_NOMEM, "cudaMalloc of " + std::to_string(bytes) + " bytes failed: " + cudaGetErrorString(e));
  return CUBE_OK;
}

// dense n^3 <-> padded n^3 (row stride n+2), device to device
int to_padded(cube_dpm* d, float* dst, const float* src, int n) {
  cube_ctx* c = &d->base;
  const size_t row = sizeof(float) * n;
  CUBE_CUDA(c, cudaMemcpy2DAsync(dst, row + 8, src, row, row, (size_t)n * n, cudaMemcpyDeviceToDevice, c->stream));
  return CUBE_OK;
}
int from_padded(cube_dpm* d, float* dst, const float* src, int n) {
  cube_ctx* c = &d->base;
  const size_t row = sizeof(float) * n;
  CUBE_CUDA(c, cudaMemcpy2DAsync(dst, row, src, row + 8, row, (size_t)n * n, cudaMemcpyDeviceToDevice, c->stream));
  return CUBE_OK;
}

int ready(cube_dpm* d) {
  if (!d) return CUBE_ERR_ARG;
  CUBE_CUDA(&d->base, cudaSetDevice(d->base.device));
  return CUBE_OK;
}

}  // namespace

extern "C" int cube_dpm_create(const cube_dpm_params* p, const cube_cosmology* cs, int device, cube_dpm** out) {
  if (!p || !cs || !out) return CUBE_ERR_ARG;
  *out = nullptr;
  cube_dpm* d = new (std::nothrow) cube_dpm();
  if (!d) return CUBE_ERR_NOMEM;
  *out = d;
  d->p = *p;
  d->base.device = device;
  if (p->ng < 16 || p->ng % 2 || p->npd < 16 || p->npd % 2 || p->ng % p->npd)
    return dpm_fail(d, CUBE_ERR_ARG, "ng and npd must be even, at least 16, and npd must divide ng");
  if (p->max_steps < 1 || p->ckpt_every < 1) return dpm_fail(d, CUBE_ERR_ARG, "max_steps and ckpt_every must be positive");
  if (!(cs->box > 0.f)) return dpm_fail(d, CUBE_ERR_ARG, "box must be positive");
  d->ng = p->ng;
  d->npd = p->npd;
  d->step = p->ng / p->npd;
  d->lat_ = Lattice{d->npd, d->step, d->ng, make_fastdiv((uint32_t)d->npd)};
  d->np = (int64_t)p->npd * p->npd * p->npd;
  d->mass = (float)((double)p->ng * p->ng * p->ng / (double)d->np);  // mean density 1 per cell
  const double a = 1.0 / (1.0 + (double)p->z_init);
  d->vf = (float)cube_ic_vfactor(a, cs->omega_m, cs->omega_l);
  cube_ctx* c = &d->base;
  CUBE_CUDA(c, cudaSetDevice(device));
  CUBE_CUDA(c, cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
  for (cudaEvent_t& e : d->ev) CUBE_CUDA(c, cudaEventCreate(&e));
  const size_t sb = sizeof(float) * 3 * (size_t)d->np;
  const int ns = (p->max_steps + p->ckpt_every - 1) / p->ckpt_every;
  int r;
  if ((r = dalloc(d, &d->green, sizeof(float) * spec_count(d->ng))) || (r = dalloc(d, &d->filt, sizeof(float) * spec_count(d->npd))) ||
      (r = dalloc(d, &d->mesh, pad_bytes(d->ng))) || (r = dalloc(d, &d->adj, pad_bytes(d->ng))) ||
      (r = dalloc(d, &d->lat, pad_bytes(d->npd))) || (r = dalloc(d, &d->x, sb)) || (r = dalloc(d, &d->v, sb)) ||
      (r = dalloc(d, &d->gx, sb)) || (r = dalloc(d, &d->gv, sb)) || (r = dalloc(d, &d->seg, 2 * sb * ns)) ||
      (r = dalloc(d, &d->pos, sb * p->ckpt_every)) || (r = dalloc(d, &d->phis, pad_bytes(d->ng) * p->ckpt_every)) ||
      (r = dalloc(d, reinterpret_cast<float**>(&d->fix), sizeof(long long) * (size_t)d->ng * d->ng * d->ng)) ||
      (r = dalloc(d, reinterpret_cast<float**>(&d->gmax), sizeof(unsigned int))))
    return r;
  CUBE_CUDA(c, cudaMemsetAsync(d->fix, 0, sizeof(long long) * (size_t)d->ng * d->ng * d->ng, c->stream));
  // deposit sums stay below 2^61: mass * np < 2^(ilogb + 1)
  d->dep_shift = 60 - std::ilogb((double)d->mass * (double)d->np);
  if ((r = make_plan(d, &d->pm_r2c, d->ng, CUFFT_R2C)) || (r = make_plan(d, &d->pm_c2r, d->ng, CUFFT_C2R)) ||
      (r = make_plan(d, &d->ic_r2c, d->npd, CUFFT_R2C)) || (r = make_plan(d, &d->ic_c2r, d->npd, CUFFT_C2R)))
    return r;
  k_dpm_green<<<cube_grid((int64_t)spec_count(d->ng), 256), 256, 0, c->stream>>>(d->green, d->ng);
  CUBE_CUDA(c, cudaGetLastError());
  // the IC filter on the lattice; the kernel spectrum is staged in lat, the
  // Delta^2 tables in adj
  r = cube_ic_filter(c, *cs, a, d->npd, d->ic_r2c, d->ic_c2r, d->lat, d->adj, d->filt);
  if (r) return r;
  CUBE_CUDA(c, cudaStreamSynchronize(c->stream));
  return CUBE_OK;
}

extern "C" int cube_dpm_destroy(cube_dpm* d) {
  if (!d) return CUBE_ERR_ARG;
  release(d);
  delete d;
  return CUBE_OK;
}

extern "C" const char* cube_dpm_last_error(const cube_dpm* d) { return d ? d->base.err.c_str() : "null context"; }

extern "C" void* cube_dpm_stream(cube_dpm* d) { return d ? (void*)d->base.stream : nullptr; }

extern "C" int64_t cube_dpm_nparticles(const cube_dpm* d) { return d ? d->np : -1; }

extern "C" int cube_dpm_set_schedule(cube_dpm* d, int nsteps, const float* drift, const float* kick) {
  int r = ready(d);
  if (r) return r;
  if (nsteps < 1 || nsteps > d->p.max_steps || !drift || !kick)
    return dpm_fail(d, CUBE_ERR_ARG, "schedule needs 1..max_steps drift and kick coefficients");
  d->drift.assign(drift, drift + nsteps);
  d->kick.assign(kick, kick + nsteps);
  d->nsteps = nsteps;
  drop_graphs(d);
  d->nforward = 0;
  return CUBE_OK;
}

extern "C" int cube_dpm_noise(cube_dpm* d, uint32_t seed, float* noise) {
  int r = ready(d);
  if (r) return r;
  if (!noise) return CUBE_ERR_ARG;
  cube_ic_noise(noise, d->npd, d->npd, seed, d->base.stream);
  CUBE_CUDA(&d->base, cudaGetLastError());
  CUBE_CUDA(&d->base, cudaStreamSynchronize(d->base.stream));
  return CUBE_OK;
}

extern "C" int cube_dpm_forward(cube_dpm* d, const float* noise, float* x, float* v) {
  int r = ready(d);
  if (r) return r;
  if (!noise || !x || !v) return CUBE_ERR_ARG;
  if (!d->nsteps) return dpm_fail(d, CUBE_ERR_STATE, "no schedule set");
  cube_ctx* c = &d->base;
  if (!d->gfwd && (r = capture(d, record_forward, &d->gfwd))) return r;
  if ((r = to_padded(d, d->lat, noise, d->npd))) return r;
  CUBE_CUDA(c, cudaEventRecord(d->ev[0], c->stream));
  CUBE_CUDA(c, cudaGraphLaunch(d->gfwd, c->stream));
  CUBE_CUDA(c, cudaEventRecord(d->ev[1], c->stream));
  const size_t sb = sizeof(float) * 3 * (size_t)d->np;
  CUBE_CUDA(c, cudaMemcpyAsync(x, d->x, sb, cudaMemcpyDeviceToDevice, c->stream));
  CUBE_CUDA(c, cudaMemcpyAsync(v, d->v, sb, cudaMemcpyDeviceToDevice, c->stream));
  CUBE_CUDA(c, cudaStreamSynchronize(c->stream));
  CUBE_CUDA(c, cudaEventElapsedTime(&d->fwd_ms, d->ev[0], d->ev[1]));
  d->nforward++;
  return CUBE_OK;
}

extern "C" int cube_dpm_backward(cube_dpm* d, const float* gx, const float* gv, float* gnoise, float* gx0,
                                 float* gv0) {
  int r = ready(d);
  if (r) return r;
  if (!gx || !gv || !gnoise) return CUBE_ERR_ARG;
  if (!d->nforward) return dpm_fail(d, CUBE_ERR_STATE, "backward needs a forward pass with this schedule");
  cube_ctx* c = &d->base;
  if (!d->gbwd && (r = capture(d, record_backward, &d->gbwd))) return r;
  const size_t sb = sizeof(float) * 3 * (size_t)d->np;
  CUBE_CUDA(c, cudaMemcpyAsync(d->gx, gx, sb, cudaMemcpyDeviceToDevice, c->stream));
  CUBE_CUDA(c, cudaMemcpyAsync(d->gv, gv, sb, cudaMemcpyDeviceToDevice, c->stream));
  CUBE_CUDA(c, cudaEventRecord(d->ev[2], c->stream));
  CUBE_CUDA(c, cudaGraphLaunch(d->gbwd, c->stream));
  CUBE_CUDA(c, cudaEventRecord(d->ev[3], c->stream));
  if ((r = from_padded(d, gnoise, d->lat, d->npd))) return r;
  if (gx0) CUBE_CUDA(c, cudaMemcpyAsync(gx0, d->gx, sb, cudaMemcpyDeviceToDevice, c->stream));
  if (gv0) CUBE_CUDA(c, cudaMemcpyAsync(gv0, d->gv, sb, cudaMemcpyDeviceToDevice, c->stream));
  CUBE_CUDA(c, cudaStreamSynchronize(c->stream));
  CUBE_CUDA(c, cudaEventElapsedTime(&d->bwd_ms, d->ev[2], d->ev[3]));
  return CUBE_OK;
}

extern "C" int cube_dpm_density(cube_dpm* d, const float* x, float* rho) {
  int r = ready(d);
  if (r) return r;
  if (!x || !rho) return CUBE_ERR_ARG;
  if ((r = deposit(d, x, nullptr, 0.f, nullptr, nullptr))) return r;
  if ((r = from_padded(d, rho, d->mesh, d->ng))) return r;
  CUBE_CUDA(&d->base, cudaStreamSynchronize(d->base.stream));
  return CUBE_OK;
}

extern "C" int cube_dpm_density_adjoint(cube_dpm* d, const float* x, const float* grho, float* gx) {
  int r = ready(d);
  if (r) return r;
  if (!x || !grho || !gx) return CUBE_ERR_ARG;
  cube_ctx* c = &d->base;
  if ((r = to_padded(d, d->adj, grho, d->ng))) return r;
  k_dpm_deposit_adj<<<cube_grid(d->np, 256), 256, 0, c->stream>>>(x, d->np, d->lat_, d->adj, d->mass, 0.f, gx, nullptr,
                                                                   0);
  CUBE_CUDA(c, cudaGetLastError());
  CUBE_CUDA(c, cudaStreamSynchronize(c->stream));
  return CUBE_OK;
}

extern "C" int cube_dpm_tables(cube_dpm* d, float* ic_filter, float* green) {
  int r = ready(d);
  if (r) return r;
  cube_ctx* c = &d->base;
  if (ic_filter)
    CUBE_CUDA(c, cudaMemcpyAsync(ic_filter, d->filt, sizeof(float) * spec_count(d->npd), cudaMemcpyDeviceToHost, c->stream));
  if (green)
    CUBE_CUDA(c, cudaMemcpyAsync(green, d->green, sizeof(float) * spec_count(d->ng), cudaMemcpyDeviceToHost, c->stream));
  CUBE_CUDA(c, cudaStreamSynchronize(c->stream));
  return CUBE_OK;
}

extern "C" int cube_dpm_info(const cube_dpm* d, float* mass, float* vf, float* fwd_ms, float* bwd_ms) {
  if (!d) return CUBE_ERR_ARG;
  if (mass) *mass = d->mass;
  if (vf) *vf = d->vf;
  if (fwd_ms) *fwd_ms = d->fwd_ms;
  if (bwd_ms) *bwd_ms = d->bwd_ms;
  return CUBE_OK;
}
