// cube_pm.cu -- particle_mesh (pm.f90:2-415) on one GB300.
//
// Fine level: one periodic nf^3 mesh (nf = nc*ncell) instead of the
// reference's nnt^3 tile boxes of nfe^3: the fine kernel is the 31^3 table
// (offsets -15..15 < nfb=24), so the force on each tile's physical region is
// the same linear convolution either way; the global mesh does (nf/nft)^3
// fewer cells of FFT work and needs no buffer deposit.
//   deposit (CIC, tile-local real(4) tempx as pm.f90:63) -> cuFFT R2C ->
//   multiply by i*K_d (pm.f90:119-120) -> 3 x cuFFT C2R -> f2 max -> kick
//   (pm.f90:129-189, decode sigma_vi, encode sigma_vi_new).
// Coarse level: nc^3 periodic mesh, deposit with the -0.5 shift
// (pm.f90:221), R2C, i*K_c, C2R, kick (pm.f90:322-387) with vmax.
// The 1/n^3 normalisation is folded into the stored kernels.
#include <cmath>
#include <vector>

#include "cube_internal.cuh"

namespace {

// ----------------------------------------------------------- Green's functions
// odd-mirrored fine table in the periodic nf^3 box (kernel_f.f90:25-31)
__global__ void k_fill_fine_table(const float* __restrict__ tab, int nfc, int pp_zero, int dim, int nf,
                                  float* __restrict__ box) {
  int w = 2 * nfc - 1;
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= w * w * w) return;
  int ox = t % w - (nfc - 1), oy = (t / w) % w - (nfc - 1), oz = t / (w * w) - (nfc - 1);
  int ax = abs(ox), ay = abs(oy), az = abs(oz);
  float v = tab[ax + nfc * (ay + nfc * (az + nfc * dim))];  // fk_table(i,j,k,d)
  if (ax <= pp_zero && ay <= pp_zero && az <= pp_zero) v = 0.f;
  int neg = dim == 0 ? ox < 0 : (dim == 1 ? oy < 0 : oz < 0);
  if (neg) v = -v;
  box[mesh_idx(nf, wrapi(ox, nf), wrapi(oy, nf), wrapi(oz, nf))] = v;
}

// kern[idx] = Im(fft)[idx] * scale
__global__ void k_take_imag(const float2* __restrict__ spec, int64_t n, float scale, float* __restrict__ kern) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    kern[i] = spec[i].y * scale;
}

// LRCKCORR (kernel_c.f90:102-116): for |k|<=8 and k_d != 0 replace K by
// K*0.25*pi*ksin_d/sum(ksin^2)/Im(FFT(raw)).  At nc = 16 the sphere reaches the
// Nyquist plane, where the odd raw kernel's transform is exactly zero and the
// reference would divide 0 by 0; there K keeps its value (also zero).
__global__ void k_lrck(float* __restrict__ kern, const float2* __restrict__ raw, int nc, int dim) {
  int nh = nc / 2 + 1;
  int64_t n = (int64_t)nh * nc * nc;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    int ix = (int)(i % nh), iy = (int)((i / nh) % nc), iz = (int)(i / ((int64_t)nh * nc));
    float k[3];
    k[0] = (float)(((ix + nc / 2) % nc) - nc / 2);
    k[1] = (float)(((iy + nc / 2) % nc) - nc / 2);
    k[2] = (float)(((iz + nc / 2) % nc) - nc / 2);
    float kr = sqrtf(k[0] * k[0] + k[1] * k[1] + k[2] * k[2]);
    if (kr > 8.0f || k[dim] == 0.f) continue;
    float s[3];
    for (int d = 0; d < 3; d++) s[d] = 2.f * sinf(CUBE_PI_F * k[d] / (float)nc);
    float ss = (s[0] * s[0] + s[1] * s[1]) + s[2] * s[2];
    if (raw[i].y == 0.f) continue;
    float v = kern[i];
    v = v * 0.25f;
    v = v * CUBE_PI_F;
    v = v * s[dim];
    v = v / ss;
    v = v / raw[i].y;
    kern[i] = v;
  }
}

__global__ void k_scale(float* __restrict__ a, int64_t n, float s) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    a[i] *= s;
}

// ---------------------------------------------------------------- deposit
// Deterministic CIC deposit.  One CTA owns a brick of BX x BY x BZ coarse
// cells and every mesh cell inside it: it reads the particles of the brick's
// coarse cells and of the LO/HI neighbouring layers whose CIC stencils reach
// into it (fine mesh: the +1 spill of the layer below; coarse mesh with its
// -0.5 shift: one layer on each side), accumulates the weights in shared
// memory as 2^-32 fixed point with 64-bit integer atomics (integer addition is
// associative, so the sum does not depend on thread order), and writes each
// owned cell once.  No memset, no global atomics, bitwise reproducible.
// The weights are the reference's real(4) products (pm.f90:63-77, 221-233),
// computed from tempx in the tile-local frame.
struct DepArgs {
  Geo g;
  const void* xp;
  const int32_t* rhoc;
  const int64_t* cstart;
  float mass;
  float* rho;                 // padded periodic mesh, row stride n+2
  unsigned long long* total;  // sum of all owned cells in fixed point (exact)
  int ng;                     // power-spectrum mesh (kPk only)
  float qscale, qinv;         // fixed-point scale 2^s and 2^-s (dep_shift)
  int accumulate;             // add to the mesh (a second species) instead of writing it
};



// kPk: the power-spectrum deposit of cicpower.f90:100-133 (position
// (cell + frac)*ng/nc - 0.5 in real(4), global frame) instead of the PM ones
template <int MPC, int BX, int BY, int BZ, int LO, int HI, bool kPk = false>
__global__ void __launch_bounds__(256) k_deposit_det(DepArgs a) {
  constexpr int SX = BX + LO + HI, SY = BY + LO + HI, SZ = BZ + LO + HI;
  constexpr int NSRC = SX * SY * SZ;
  constexpr int MX = MPC * BX, MY = MPC * BY, MZ = MPC * BZ;
  extern __shared__ __align__(16) unsigned acc[];  // low words [0, MX*MY*MZ), carry words after them
  unsigned* carry = acc + MX * MY * MZ;
  __shared__ int pref[NSRC];
  __shared__ long long sstart[NSRC];
  // kAxis: the fine deposit tests the stencil per axis (a 2-bit mask each,
  // the whole stencil skipped when one is empty) and shares the x*y weight
  // products between z's two corners; the coarse deposit, whose stencils more
  // often straddle the brick's edge, measured faster with the plain per-corner
  // test (0.21 ms of 2.70 at 512^3), the fine one slower (0.37 ms of 5.54)
  constexpr bool kAxis = MPC > 1;
  // per source cell, 16 bits a dimension: the 1-based tile-local coordinate
  // (kPk: the global coarse coordinate) that the particle's frame needs
  __shared__ unsigned long long sframe[NSRC];
  __shared__ unsigned long long btot;
  const Geo& g = a.g;
  const int nc = g.nc, n = kPk ? a.ng : (MPC == 1 ? g.nc : g.nf);
  int nbx = (nc + BX - 1) / BX, nby = (nc + BY - 1) / BY;
  int b = blockIdx.x;
  int C0[3] = {(b % nbx) * BX, ((b / nbx) % nby) * BY, (b / (nbx * nby)) * BZ};
  int B[3] = {min(BX, nc - C0[0]), min(BY, nc - C0[1]), min(BZ, nc - C0[2])};
  // 2*MX*MY*MZ is a multiple of 4: 16-byte stores
  for (int i = 4 * threadIdx.x; i < 2 * MX * MY * MZ; i += 4 * blockDim.x)
    *reinterpret_cast<uint4*>(acc + i) = make_uint4(0u, 0u, 0u, 0u);
  if (threadIdx.x == 0) btot = 0ull;
  // source cells, their particle counts and frames
  for (int t = threadIdx.x; t < NSRC; t += blockDim.x) {
    const int sl[3] = {t % SX - LO, (t / SX) % SY - LO, t / (SX * SY) - LO};
    int cnt = 0;
    long long st = 0;
    unsigned long long fr = 0;
    if (sl[0] < B[0] + HI && sl[1] < B[1] + HI && sl[2] < B[2] + HI) {
      int gc[3];
#pragma unroll
      for (int d = 0; d < 3; d++) {
        gc[d] = wrap1(C0[d] + sl[d], nc);
        int Tq, L;
        tile_local(g, gc[d], Tq, L);
        fr |= (unsigned long long)(unsigned)(kPk ? gc[d] : L) << (16 * d);
      }
      int64_t c = cell_id(g, gc[0], gc[1], gc[2]);
      cnt = a.rhoc[c];
      st = a.cstart[c];
    }
    pref[t] = cnt;
    sstart[t] = st;
    sframe[t] = fr;
  }
  __syncthreads();
  const int total = block_exclusive_scan(pref, NSRC);
  const int lim[3] = {MPC * B[0], MPC * B[1], MPC * B[2]};
  for_box_particles<SX>(pref, sstart, SX, SY * SZ, total, [&](int64_t p, int sxi, int row) {
    const int sl[3] = {sxi - LO, row % SY - LO, row / SY - LO};
    const unsigned long long fr = sframe[sxi + SX * row];
    int rel[3];
    unsigned ok[3];  // bit o: mesh index rel + o lies in the brick
    float d1[3], d2[3];
#pragma unroll
    for (int d = 0; d < 3; d++) {
      const int v = (int)((fr >> (16 * d)) & 0xffffu);  // L, or kPk the global coordinate
      int code = load_code(a.xp, 3 * p + d, g.izipx);
      float tx;
      if (kPk) {
        float frac = __fmul_rn(pos_off_f(code, g.izipx), g.izipx == 1 ? 1.0f / 256.0f : 1.0f / 65536.0f);
        // the particle's own global frame, as the reference rounds it
        float pos = __fadd_rn((float)v, frac);
        tx = __fsub_rn(__fdiv_rn(__fmul_rn(pos, (float)a.ng), (float)nc), 0.5f);
      } else {
        tx = MPC == 1 ? coarse_tempx(v, code, g.izipx) : fine_tempx(MPC, v, code, g.izipx);
      }
      float fl = floorf(tx);
      d1[d] = __fsub_rn(__fadd_rn(fl, 1.0f), tx);
      d2[d] = __fsub_rn(1.0f, d1[d]);
      // mesh index relative to the brick
      // (kPk: unwrap the ring cell's periodic image, then relative to the brick)
      rel[d] = kPk ? (int)fl + MPC * (sl[d] - v) : MPC * sl[d] + (int)fl - MPC * (v - 1);
      ok[d] = (unsigned)(rel[d] >= 0 && rel[d] < lim[d]) | ((unsigned)(rel[d] >= -1 && rel[d] + 1 < lim[d]) << 1);
    }
    if (kAxis && !(ok[0] && ok[1] && ok[2])) return;  // the whole stencil lies outside the brick
    // the reference's product order ((d_x * d_y) * d_z) * mass
    float wxy[4];
#pragma unroll
    for (int k = 0; k < 4; k++) wxy[k] = kAxis ? __fmul_rn(k & 1 ? d2[0] : d1[0], k & 2 ? d2[1] : d1[1]) : 0.f;
    const int e0 = rel[0] + MX * (rel[1] + MY * rel[2]);
#pragma unroll
    for (int k = 0; k < 8; k++) {
      const int ox = k & 1, oy = (k >> 1) & 1, oz = k >> 2;
      if (kAxis) {
        if (!((ok[0] >> ox) & (ok[1] >> oy) & (ok[2] >> oz) & 1u)) continue;
      } else {
        const int x = rel[0] + ox, y = rel[1] + oy, z = rel[2] + oz;
        if (x < 0 || y < 0 || z < 0 || x >= lim[0] || y >= lim[1] || z >= lim[2]) continue;
      }
      const float wxyk = kAxis ? wxy[k & 3] : __fmul_rn(ox ? d2[0] : d1[0], oy ? d2[1] : d1[1]);
      float w = __fmul_rn(__fmul_rn(wxyk, oz ? d2[2] : d1[2]), a.mass);
      // w * 2^s (exact scaling, truncated) < 2^31; carry out of the low word
      const unsigned q = __float2uint_rz(__fmul_rn(w, a.qscale));
      const int e = kAxis ? e0 + ox + MX * (oy + MY * oz) : (rel[0] + ox) + MX * ((rel[1] + oy) + MY * (rel[2] + oz));
      const unsigned old = atomicAdd(&acc[e], q);
      if (old + q < old) atomicAdd(&carry[e], 1u);
    }
  });
  __syncthreads();
  unsigned long long mysum = 0;
  // (hi*2^32 + lo) * 2^-s as float
  const float qhi = __fmul_rn(a.qinv, 4294967296.0f);
  if (kAxis) {
    // KX neighbouring x cells a thread, written as KX/2 pairs: KX divides
    // MPC, so MX and the brick's extent MPC*B[0] are multiples of KX, and n
    // is even, so x starts an 8-byte aligned stretch of the padded mesh
    // (row stride n+2)
    constexpr int KX = MPC >= 4 ? 4 : 2;
    for (int i = KX * threadIdx.x; i < MX * MY * MZ; i += KX * blockDim.x) {
      const int x = i % MX, y = (i / MX) % MY, z = i / (MX * MY);
      if (x >= MPC * B[0] || y >= MPC * B[1] || z >= MPC * B[2]) continue;
      unsigned lo[KX], hi[KX];
      if constexpr (KX == 4) {
        const uint4 l = *reinterpret_cast<const uint4*>(acc + i), h = *reinterpret_cast<const uint4*>(carry + i);
        lo[0] = l.x, lo[1] = l.y, lo[2] = l.z, lo[3] = l.w;
        hi[0] = h.x, hi[1] = h.y, hi[2] = h.z, hi[3] = h.w;
      } else {
        const uint2 l = *reinterpret_cast<const uint2*>(acc + i), h = *reinterpret_cast<const uint2*>(carry + i);
        lo[0] = l.x, lo[1] = l.y;
        hi[0] = h.x, hi[1] = h.y;
      }
      float2* cell = reinterpret_cast<float2*>(a.rho + mesh_idx(n, MPC * C0[0] + x, MPC * C0[1] + y, MPC * C0[2] + z));
#pragma unroll
      for (int q = 0; q < KX / 2; q++) {
        mysum += (((unsigned long long)hi[2 * q] << 32) | lo[2 * q]) +
                 (((unsigned long long)hi[2 * q + 1] << 32) | lo[2 * q + 1]);
        float2 r = make_float2(__fmaf_rn((float)lo[2 * q], a.qinv, __fmul_rn((float)hi[2 * q], qhi)),
                               __fmaf_rn((float)lo[2 * q + 1], a.qinv, __fmul_rn((float)hi[2 * q + 1], qhi)));
        if (a.accumulate) {
          const float2 o = cell[q];
          r = make_float2(__fadd_rn(o.x, r.x), __fadd_rn(o.y, r.y));
        }
        cell[q] = r;
      }
    }
  } else {
    for (int i = threadIdx.x; i < MX * MY * MZ; i += blockDim.x) {
      const int x = i % MX, y = (i / MX) % MY, z = i / (MX * MY);
      if (x >= MPC * B[0] || y >= MPC * B[1] || z >= MPC * B[2]) continue;
      const unsigned lo = acc[i], hi = carry[i];
      mysum += ((unsigned long long)hi << 32) | lo;
      float r = __fmaf_rn((float)lo, a.qinv, __fmul_rn((float)hi, qhi));
      float* cell = a.rho + mesh_idx(n, MPC * C0[0] + x, MPC * C0[1] + y, MPC * C0[2] + z);
      *cell = a.accumulate ? __fadd_rn(*cell, r) : r;
    }
  }
  for (int o = 16; o > 0; o >>= 1) mysum += __shfl_xor_sync(0xffffffffu, mysum, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(&btot, mysum);
  __syncthreads();
  if (threadIdx.x == 0 && a.total) atomicAdd(a.total, btot);
}

template <int MPC, int BX, int BY, int BZ, int LO, int HI, bool kPk = false>
int launch_deposit(cube_ctx* c, const DepArgs& a) {
  int nc = c->p.nc;
  int nb = ((nc + BX - 1) / BX) * ((nc + BY - 1) / BY) * ((nc + BZ - 1) / BZ);
  size_t smem = 2 * sizeof(unsigned) * (MPC * BX) * (MPC * BY) * (MPC * BZ);
  auto kern = k_deposit_det<MPC, BX, BY, BZ, LO, HI, kPk>;
  CUBE_CUDA(c, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  kern<<<nb, 256, smem, c->stream>>>(a);
  CUBE_CUDA(c, cudaGetLastError());
  return CUBE_OK;
}

// The deposits' brick shapes (cube_set_option CUBE_OPT_DEPOSIT_FINE / _COARSE):
// larger bricks re-read fewer neighbour particles, smaller ones hold less
// shared memory per CTA (more CTAs per SM) and give small meshes more CTAs.
// Every shape writes the same exact fixed-point sums.
int launch_fine_deposit(cube_ctx* c, const DepArgs& a) {
  switch (c->opt_dep_fine) {
    case 1: return launch_deposit<4, 4, 4, 4, 1, 0>(c, a);  // 16^3 fine cells, 32 KB
    case 2: return launch_deposit<4, 8, 4, 2, 1, 0>(c, a);  // 32x16x8, 32 KB
    case 3: return launch_deposit<4, 4, 4, 2, 1, 0>(c, a);  // 16x16x8, 16 KB
    default: return launch_deposit<4, 8, 4, 4, 1, 0>(c, a);  // 32x16x16, 64 KB
  }
}
int launch_coarse_deposit(cube_ctx* c, const DepArgs& a) {
  switch (c->opt_dep_coarse) {
    case 1: return launch_deposit<1, 16, 8, 8, 1, 1>(c, a);
    case 2: return launch_deposit<1, 8, 8, 4, 1, 1>(c, a);
    case 3: return launch_deposit<1, 4, 4, 4, 1, 1>(c, a);
    default: return launch_deposit<1, 8, 8, 8, 1, 1>(c, a);
  }
}

// ------------------------------------------------------- spectral multiply
// out_d = i*K_d*rho_k for the three components in one pass (pm.f90:119-120)
__global__ void k_green3(const float2* __restrict__ rk, const float* __restrict__ kern, int64_t n,
                         float2* __restrict__ o0, float2* __restrict__ o1, float2* __restrict__ o2) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    float2 r = rk[i];
    float k0 = kern[i], k1 = kern[n + i], k2 = kern[2 * n + i];
    o0[i] = make_float2(-r.y * k0, r.x * k0);
    o1[i] = make_float2(-r.y * k1, r.x * k1);
    o2[i] = make_float2(-r.y * k2, r.x * k2);
  }
}

// maxval(sum(force**2,1)) over the mesh (pm.f90:126, 315): one block per row
// (y, z) at a time, float2 loads along x (rows start 8-byte aligned: stride n+2)
__device__ __forceinline__ float f2sum(float a, float b, float c) {
  return __fadd_rn(__fadd_rn(__fmul_rn(a, a), __fmul_rn(b, b)), __fmul_rn(c, c));
}
// kPre: then rewrite each force value as its kick factor force*a_mid*dt/6/pi
template <bool kPre>
__global__ void k_f2max(float* __restrict__ f0, float* __restrict__ f1, float* __restrict__ f2, int n,
                        unsigned int* __restrict__ out, float a_mid, float dt, const StepDev* sd) {
  if (sd) {  // graph mode
    a_mid = sd->h.a_mid;
    dt = sd->h.dt;
  }
  const int64_t rows = (int64_t)n * n;
  const int h = n >> 1;
  float m = 0.f;
  for (int64_t r = blockIdx.x; r < rows; r += gridDim.x) {
    const int64_t o = r * (n + 2);
    float2* a = reinterpret_cast<float2*>(f0 + o);
    float2* b = reinterpret_cast<float2*>(f1 + o);
    float2* c = reinterpret_cast<float2*>(f2 + o);
    for (int x = threadIdx.x; x < h; x += blockDim.x) {
      float2 u = a[x], v = b[x], w = c[x];
      m = fmaxf(m, fmaxf(f2sum(u.x, v.x, w.x), f2sum(u.y, v.y, w.y)));
      if (kPre) {
        a[x] = make_float2(kick_pre(u.x, a_mid, dt), kick_pre(u.y, a_mid, dt));
        b[x] = make_float2(kick_pre(v.x, a_mid, dt), kick_pre(v.y, a_mid, dt));
        c[x] = make_float2(kick_pre(w.x, a_mid, dt), kick_pre(w.y, a_mid, dt));
      }
    }
    if ((n & 1) && threadIdx.x == 0) {
      const int64_t e = o + n - 1;
      m = fmaxf(m, f2sum(f0[e], f1[e], f2[e]));
      if (kPre) {
        f0[e] = kick_pre(f0[e], a_mid, dt);
        f1[e] = kick_pre(f1[e], a_mid, dt);
        f2[e] = kick_pre(f2[e], a_mid, dt);
      }
    }
  }
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomic_max_pos(out, m);
}

// ------------------------------------------------------------------- kicks
struct KickArgs {
  Geo g;
  int64_t np;
  const void* xp;
  const void* vp_in;
  void* vp_out;            // may equal vp_in (fine kick updates in place)
  const int32_t* pcell;
  const int32_t* rhoc;     // staged kernels: cell counts and starts
  const int64_t* cstart;
  const float* vfield;
  const float* f[3];
  CodecView cin, cout;     // decode with sigma_in, encode with sigma_out
  float a_mid, dt;
  unsigned int* vmax_bits; // coarse kick only: exact vmax per component
  float tau[3];            // coarse kick: lanes whose |v+vfield| may reach tau are evaluated exactly
  unsigned int* vmax_lo;   // coarse kick: the largest lower bound of |v+vfield| (certain to be <= vmax)
  int vmax_only;           // rerun for the exact vmax (write nothing): lanes whose bound reaches vmax_lo
  int exact_only;          // skip the certified fast path
  unsigned long long* nexact;
  const StepDev* sd;       // graph mode: a_mid, dt, tau from the device
  unsigned int* vmax_est;        // fine kick: record max |v + vfield| (FP32) here when set
  const unsigned int* tau_est;   // coarse kick: tau = 0.7 of this estimate when set
  const float* fpp;              // fine kick: when set, first the PP kick by these pair forces
  float pp_kf;                   // its factor a_mid*dt/6/pi, float and double
  double pp_kd;
  const unsigned* pp_act;        // PP prefilter: set bits are the particles PP has kicked, the others take zero kicks
};
__device__ __forceinline__ float kick_amid(const KickArgs& a) { return a.sd ? __ldg(&a.sd->h.a_mid) : a.a_mid; }
__device__ __forceinline__ float kick_dt(const KickArgs& a) { return a.sd ? __ldg(&a.sd->h.dt) : a.dt; }
__device__ __forceinline__ float kick_tau(const KickArgs& a, int d) {
  if (a.sd) return __ldg(&a.sd->h.tau[d]);
  return a.tau_est ? __fmul_rn(0.7f, __uint_as_float(__ldg(a.tau_est + d))) : a.tau[d];
}

// The kick velocity of the reference is the FP64 chain
//   v = decode; v = v + t1; ...; v = v + t8       (pm.f90:145-153)
// with t_i the real(4) CIC terms.  The fast path forms V_f = fl32(hi(decode) + S)
// with S the FP32 sum of the terms; its distance from the reference value is
// bounded by
//   gamma_7 sum|t_i| + 2^-24 (|decode| + |V_f|) + 9*2^-53 (|decode| + sum|t_i| + |V_f|)
// (recursive-summation bound, gamma_7 = 7u/(1-7u), u = 2^-24; the decode table's
// float hi is within half an ulp).  certify_abs keeps the code only when every
// double inside that bound encodes to it; otherwise the lane runs the exact
// chain, so the stored code is always the reference's.
//
// The exact chain (and, in the coarse kick, the exact |v + vfield| of lanes
// that may set vmax) is needed by a few components in a thousand, but a warp
// runs it whenever one of its 32 lanes needs it, on the FP64 pipe.  So each
// warp queues those (particle, component, code) entries in shared memory and
// runs the chain 32 entries at a time, each lane recomputing its entry's CIC
// corners and terms (the same arithmetic, the same bits).  An entry packs
// the particle index (bits 18 and up), the 16-bit code and the component.
constexpr int KICK_Q = 64;  // queue entries per warp: at most 31 pending + 32 from one component
__device__ __forceinline__ unsigned long long kick_qkey(int64_t p, int d, int code) {
  return ((unsigned long long)p << 18) | ((unsigned long long)(code & 0xffff) << 2) | (unsigned long long)d;
}

// a corner's mesh index is xo[i] + yo[j] + zo[k] (i, j, k = 0 for the lower
// corner, 1 for the upper; x and y parts in 32 bits)
struct KickCorners {
  int xo[2], yo[2];
  int64_t zo[2];
  float d1[3], d2[3];
  int64_t cell;
};

template <bool kFine>
__device__ __forceinline__ void kick_corners(const KickArgs& a, int64_t p, KickCorners& k) {
  const Geo& g = a.g;
  k.cell = a.pcell[p];
  int gc[3];
  cell_coords(g, k.cell, gc[0], gc[1], gc[2]);
  int i1[3], i2[3];
  const int n = kFine ? g.nf : g.nc;
  for (int d = 0; d < 3; d++) {
    int T, L;
    tile_local(g, gc[d], T, L);
    int code = load_code(a.xp, 3 * p + d, g.izipx);
    float tx;
    int base;
    if (kFine) {
      tx = fine_tempx(g.ncell, L, code, g.izipx);  // tile-local frame (pm.f90:138)
      base = T * g.nt * g.ncell + (int)floorf(tx);
    } else {
      tx = coarse_tempx(gc[d] + 1, code, g.izipx);  // global frame (pm.f90:335)
      base = (int)floorf(tx);
    }
    float fl = floorf(tx);
    k.d1[d] = __fsub_rn(__fadd_rn(fl, 1.0f), tx);
    k.d2[d] = __fsub_rn(1.0f, k.d1[d]);
    i1[d] = wrap1(base, n);
    i2[d] = wrap1(base + 1, n);
  }
  // mesh_idx(n, x, y, z) = x + (n+2)*(y + n*z)
  k.xo[0] = i1[0];
  k.xo[1] = i2[0];
  k.yo[0] = (n + 2) * i1[1];
  k.yo[1] = (n + 2) * i2[1];
  k.zo[0] = (int64_t)(n + 2) * n * i1[2];
  k.zo[1] = (int64_t)(n + 2) * n * i2[2];
}

// the eight real(4) CIC terms of component d, in the reference's order
template <bool kPre>
__device__ __forceinline__ void kick_terms(const KickArgs& a, const KickCorners& k, int d, float t[8]) {
  const float* F = a.f[d];
  const float* d1 = k.d1;
  const float* d2 = k.d2;
#define KT(c, wa, wb, wc) (kPre ? kick_w(__ldg(F + (c)), wa, wb, wc) : kick_term(__ldg(F + (c)), kick_amid(a), kick_dt(a), wa, wb, wc))
  // corners c111, c211, c121, c112, c122, c212, c221, c222
  const float* F0 = F + k.zo[0];
  const float* F1 = F + k.zo[1];
  t[0] = KT(k.xo[0] + k.yo[0] + (F0 - F), d1[0], d1[1], d1[2]);
  t[1] = KT(k.xo[1] + k.yo[0] + (F0 - F), d2[0], d1[1], d1[2]);
  t[2] = KT(k.xo[0] + k.yo[1] + (F0 - F), d1[0], d2[1], d1[2]);
  t[3] = KT(k.xo[0] + k.yo[0] + (F1 - F), d1[0], d1[1], d2[2]);
  t[4] = KT(k.xo[0] + k.yo[1] + (F1 - F), d1[0], d2[1], d2[2]);
  t[5] = KT(k.xo[1] + k.yo[0] + (F1 - F), d2[0], d1[1], d2[2]);
  t[6] = KT(k.xo[1] + k.yo[1] + (F0 - F), d2[0], d2[1], d1[2]);
  t[7] = KT(k.xo[1] + k.yo[1] + (F1 - F), d2[0], d2[1], d2[2]);
#undef KT
}

// one queued component on the reference's FP64 chain: its code, and in the
// coarse kick vmax=max(vmax,abs(vreal+vfield)) (pm.f90:349) as real(4)
template <bool kFine, bool kPre>
__device__ __forceinline__ void kick_exact_entry(const KickArgs& a, unsigned long long key, float vm[3]) {
  const int64_t p = (int64_t)(key >> 18);
  const int d = (int)(key & 3ull);
  const int code = (int)(int16_t)(uint16_t)((key >> 2) & 0xffffull);
  KickCorners k;
  kick_corners<kFine>(a, p, k);
  float t[8];
  kick_terms<kPre>(a, k, d, t);
  double v = codec_decode(a.cin, code);
  for (int i = 0; i < 8; i++) v = __dadd_rn(v, (double)t[i]);
  if (!kFine) {
    const double w = fabs(__dadd_rn(v, (double)a.vfield[3 * k.cell + d]));
    const float wf = __double2float_rn(w);
    vm[0] = d == 0 ? fmaxf(vm[0], wf) : vm[0];
    vm[1] = d == 1 ? fmaxf(vm[1], wf) : vm[1];
    vm[2] = d == 2 ? fmaxf(vm[2], wf) : vm[2];
  }
  if (!a.vmax_only) store_code(a.vp_out, 3 * p + d, a.g.izipv, codec_encode(a.cout, v));
}

// kPre: the meshes hold force*a_mid*dt/6/pi already (k_f2max<true>)
template <bool kFine, bool kPre>
__global__ void __launch_bounds__(256, 4) k_kick(KickArgs a) {
  if (a.vmax_only && a.sd) {  // graph mode: the exact vmax rerun runs only when some component needs it
    bool need = false;
    for (int d = 0; d < 3; d++)
      if (!(__uint_as_float(*(volatile unsigned int*)&a.vmax_bits[d]) >= kick_tau(a, d))) need = true;
    if (!need) return;
  }
  __shared__ unsigned long long s_q[8][KICK_Q];  // 256 threads: 8 warps
  const Geo& g = a.g;
  const int lane = threadIdx.x & 31, wq = threadIdx.x >> 5;
  int qn = 0;                      // queued entries of this warp (warp-uniform)
  float vm[3] = {0.f, 0.f, 0.f};  // coarse: exact vmax; fine: the FP32 estimate
  float vlo[3] = {0.f, 0.f, 0.f};  // coarse: lower bounds of |v + vfield|
  unsigned long long nex = 0;
  // whole warps iterate together (the queue's ballots); lanes past the end
  // compute on the last particle and store nothing
  for (int64_t p0 = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p0 - lane < a.np;
       p0 += (int64_t)gridDim.x * blockDim.x) {
    const bool valid = p0 < a.np;
    const int64_t p = valid ? p0 : a.np - 1;
    KickCorners k;
    kick_corners<kFine>(a, p, k);
    int codes[3];
#pragma unroll
    for (int d = 0; d < 3; d++) codes[d] = load_code(a.vp_in, 3 * p + d, g.izipv);
    if (kFine && a.pp_act) {
      // ext_pp_force's kick (ext_pp_force.f90:116-121) before the fine kick:
      // the prefilter's active particles were kicked by PP already; the
      // others' force is zero, their PP code the zero-kick code of theirs
      const bool on = (__ldg(a.pp_act + (p >> 5)) >> (p & 31)) & 1u;
#pragma unroll
      for (int d = 0; d < 3; d++) {
        const int z = __ldg(a.cin.rt + codes[d] + a.cin.half);
        codes[d] = on ? codes[d] : z;
      }
    } else if (kFine && a.fpp) {
      // ext_pp_force's kick before the fine kick, both in this pass: the PP
      // code (decoded and encoded with sigma_vi) is the one the fine kick decodes
      const float F[3] = {a.fpp[3 * p], a.fpp[3 * p + 1], a.fpp[3 * p + 2]};
      pp_kick3(a.cin, codes, F, a.pp_kf, a.pp_kd, a.exact_only);
    }
    for (int d = 0; d < 3; d++) {
      float t[8];
      kick_terms<kPre>(a, k, d, t);
      const int code = codes[d];
      float dh = codec_decode_ff(a.cin, code).x;
      float S = t[0], T = fabsf(t[0]);
      for (int i = 1; i < 8; i++) {
        S = __fadd_rn(S, t[i]);
        T = __fadd_rn(T, fabsf(t[i]));
      }
      float vf = __fadd_rn(dh, S);
      long long vb = f2d_bits(vf), ab = vb & 0x7fffffffffffffffLL;
      float E = 1.25f * (T * 4.76837158e-7f + (fabsf(dh) + fabsf(vf)) * 6.0e-8f + T * 1.0e-15f);
      long long nc_ = 0;
      bool ok = !a.exact_only && certify_abs(ab, E, a.cout, &nc_);
      bool need_vmax = false;
      if (!kFine) {
        const float vfd = a.vfield[3 * k.cell + d];
        // |v + vfield| of the reference's FP64 v lies in [lo, ub]
        float ub = (fabsf(vf) + E + fabsf(vfd)) * 1.000001f;
        float lo = __fmul_rn(__fsub_rn(fabsf(__fadd_rn(vf, vfd)), E), 0.99999f);
        if (valid) vlo[d] = fmaxf(vlo[d], lo);
        // the first pass: lanes that may reach tau; the rerun: lanes that may
        // reach the largest lower bound, which the maximum does
        need_vmax = ub >= (a.vmax_only ? __uint_as_float(__ldg(&a.vmax_lo[d])) : kick_tau(a, d));
      } else if (a.vmax_est && valid) {
        vm[d] = fmaxf(vm[d], fabsf(__fadd_rn(vf, a.vfield[3 * k.cell + d])));
      }
      const bool fast = ok && !need_vmax;
      if (fast && valid && !a.vmax_only) store_code(a.vp_out, 3 * p + d, g.izipv, vb < 0 ? -nc_ : nc_);
      const bool defer = valid && !fast;
      const unsigned m = __ballot_sync(0xffffffffu, defer);
      if (m) {
        if (defer) s_q[wq][qn + __popc(m & ((1u << lane) - 1u))] = kick_qkey(p, d, code);
        qn += __popc(m);
        // the chain for 32 queued entries at a time, one per lane
        if (qn >= 32) {
          __syncwarp();
          kick_exact_entry<kFine, kPre>(a, s_q[wq][qn - 32 + lane], vm);
          nex++;
          qn -= 32;
          __syncwarp();
        }
      }
    }
  }
  __syncwarp();
  if (lane < qn) {
    kick_exact_entry<kFine, kPre>(a, s_q[wq][lane], vm);
    nex++;
  }
  if (!kFine || a.vmax_est) {
    for (int d = 0; d < 3; d++) {
      float m = vm[d];
      for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
      if ((threadIdx.x & 31) == 0) atomic_max_pos(kFine ? &a.vmax_est[d] : &a.vmax_bits[d], m);
    }
  }
  if (!kFine && !a.vmax_only) {
    for (int d = 0; d < 3; d++) {
      float m = vlo[d];
      for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
      if ((threadIdx.x & 31) == 0 && m > 0.f) atomic_max_pos(&a.vmax_lo[d], m);
    }
  }
  for (int o = 16; o > 0; o >>= 1) nex += __shfl_xor_sync(0xffffffffu, nex, o);
  if ((threadIdx.x & 31) == 0 && a.nexact) atomicAdd(a.nexact, nex);
}

}  // namespace

// Fixed-point scale of the deposits: each weight w <= mass becomes the integer
// w*2^s < 2^31 with the largest such s, so a 32-bit atomic adds it (64-bit
// shared-memory atomics are several times slower); a second 32-bit counter per
// mesh point takes the carries out of the first.
int dep_shift(float mass) {
  int s = 31;
  float lim = 1.0f;
  while (lim < mass && s > 1) {
    lim *= 2.0f;
    s--;
  }
  return s;
}

// -------------------------------------------------------------- init
int cube_kernels_init(cube_ctx* c, const float* fine_table, const float* coarse_table) {
  int nf = c->nf, nc = c->p.nc, nfc = c->p.nf_cutoff;
  cudaStream_t s = c->stream;
  // ---- fine: fill the odd-mirrored table, R2C, keep Im/nf^3
  float* dtab = nullptr;
  CUBE_CUDA(c, cudaMalloc(&dtab, sizeof(float) * 3 * nfc * nfc * nfc));
  CUBE_CUDA(c, cudaMemcpyAsync(dtab, fine_table, sizeof(float) * 3 * nfc * nfc * nfc, cudaMemcpyHostToDevice, s));
  int64_t nfh = nf / 2 + 1;
  int64_t nspec = nfh * nf * (int64_t)nf;
  int64_t fpad = 2 * nspec;
  float scale_f = (float)(1.0 / ((double)nf * nf * nf));
  int w = 2 * nfc - 1;
  for (int d = 0; d < 3; d++) {
    CUBE_CUDA(c, cudaMemsetAsync(c->rho_f, 0, 4 * fpad, s));
    k_fill_fine_table<<<(w * w * w + 255) / 256, 256, 0, s>>>(dtab, nfc, c->p.pp_on ? c->p.pp_range : -1, d, nf,
                                                               c->rho_f);
    CUBE_FFT(c, cufftExecR2C(c->plan_f_r2c, c->rho_f, (cufftComplex*)c->rho_f));
    k_take_imag<<<cube_grid(nspec, 256), 256, 0, s>>>((const float2*)c->rho_f, nspec, scale_f,
                                                       c->kern_f + d * nspec);
  }
  CUBE_CUDA(c, cudaGetLastError());
  CUBE_CUDA(c, cudaStreamSynchronize(s));
  cudaFree(dtab);

  // ---- coarse: -r/r^3 with the near-field table (kernel_c.f90:16-72), on the host
  int64_t n3 = (int64_t)nc * nc * nc;
  int ncell = c->p.ncell;
  std::vector<float> ck(3 * n3), raw(3 * n3);
  auto rcoord = [&](int i) { return (float)(ncell * (((i + nc / 2) % nc) - nc / 2)); };
  for (int k = 0; k < nc; k++)
    for (int j = 0; j < nc; j++)
      for (int i = 0; i < nc; i++) {
        float rx[3] = {rcoord(i), rcoord(j), rcoord(k)};
        float r = std::sqrt(rx[0] * rx[0] + rx[1] * rx[1] + rx[2] * rx[2]);
        float r3 = (r * r) * r;
        int64_t idx = i + (int64_t)nc * (j + (int64_t)nc * k);
        for (int d = 0; d < 3; d++) raw[d * n3 + idx] = r == 0.f ? 0.f : -rx[d] / r3;
      }
  ck = raw;
  // octant copies of ck_table (kernel_c.f90:43-72); with one image all eight apply in order
  auto T = [&](int d, int i, int j, int k) { return coarse_table[d + 3 * (i + 4 * (j + 4 * k))]; };
  auto CK = [&](int d, int i, int j, int k) -> float& {  // 1-based Fortran indices into ck(d,i,j,k)
    return ck[(d - 1) * n3 + (i - 1) + (int64_t)nc * ((j - 1) + (int64_t)nc * (k - 1))];
  };
  // rev(a) maps Fortran nc-2..nc to table 4..2
  for (int k = 1; k <= 4; k++)
    for (int j = 1; j <= 4; j++)
      for (int i = 1; i <= 4; i++)
        for (int d = 1; d <= 3; d++) CK(d, i, j, k) = T(d - 1, i - 1, j - 1, k - 1);  // 1
  for (int m = 0; m < 3; m++) {  // index nc-2+m <-> table 4-m
    for (int j = 1; j <= 4; j++)
      for (int k = 1; k <= 4; k++) {
        int a = nc - 2 + m, t = 4 - m;
        // 5 x
        CK(1, a, j, k) = -T(0, t - 1, j - 1, k - 1);
        CK(2, a, j, k) = T(1, t - 1, j - 1, k - 1);
        CK(3, a, j, k) = T(2, t - 1, j - 1, k - 1);
      }
    for (int i = 1; i <= 4; i++)
      for (int k = 1; k <= 4; k++) {
        int a = nc - 2 + m, t = 4 - m;
        // 3 y
        CK(1, i, a, k) = T(0, i - 1, t - 1, k - 1);
        CK(3, i, a, k) = T(2, i - 1, t - 1, k - 1);
        CK(2, i, a, k) = -T(1, i - 1, t - 1, k - 1);
      }
    for (int i = 1; i <= 4; i++)
      for (int j = 1; j <= 4; j++) {
        int a = nc - 2 + m, t = 4 - m;
        // 2 z
        CK(1, i, j, a) = T(0, i - 1, j - 1, t - 1);
        CK(2, i, j, a) = T(1, i - 1, j - 1, t - 1);
        CK(3, i, j, a) = -T(2, i - 1, j - 1, t - 1);
      }
  }
  for (int m1 = 0; m1 < 3; m1++)
    for (int m2 = 0; m2 < 3; m2++) {
      int a1 = nc - 2 + m1, t1 = 4 - m1, a2 = nc - 2 + m2, t2 = 4 - m2;
      for (int i = 1; i <= 4; i++) {  // 4 yz: (j=a1,k=a2)
        CK(1, i, a1, a2) = T(0, i - 1, t1 - 1, t2 - 1);
        CK(2, i, a1, a2) = -T(1, i - 1, t1 - 1, t2 - 1);
        CK(3, i, a1, a2) = -T(2, i - 1, t1 - 1, t2 - 1);
      }
      for (int j = 1; j <= 4; j++) {  // 6 xz: (i=a1,k=a2)
        CK(1, a1, j, a2) = -T(0, t1 - 1, j - 1, t2 - 1);
        CK(3, a1, j, a2) = -T(2, t1 - 1, j - 1, t2 - 1);
        CK(2, a1, j, a2) = T(1, t1 - 1, j - 1, t2 - 1);
      }
      for (int k = 1; k <= 4; k++) {  // 7 xy: (i=a1,j=a2)
        CK(1, a1, a2, k) = -T(0, t1 - 1, t2 - 1, k - 1);
        CK(2, a1, a2, k) = -T(1, t1 - 1, t2 - 1, k - 1);
        CK(3, a1, a2, k) = T(2, t1 - 1, t2 - 1, k - 1);
      }
    }
  for (int m1 = 0; m1 < 3; m1++)
    for (int m2 = 0; m2 < 3; m2++)
      for (int m3 = 0; m3 < 3; m3++)  // 8 xyz
        for (int d = 1; d <= 3; d++)
          CK(d, nc - 2 + m1, nc - 2 + m2, nc - 2 + m3) = -T(d - 1, 4 - m1 - 1, 4 - m2 - 1, 4 - m3 - 1);

  // ---- FFTs and LRCKCORR; stage through force_c[0] (padded)
  int64_t nch = nc / 2 + 1;
  int64_t cspec = nch * nc * (int64_t)nc;
  float* buf = c->force_c[0];
  float* bufr = c->force_c[1];
  size_t row = (size_t)nc * 4, pitch = (size_t)(nc + 2) * 4;
  for (int d = 0; d < 3; d++) {
    CUBE_CUDA(c, cudaMemcpy2DAsync(buf, pitch, ck.data() + d * n3, row, row, (size_t)nc * nc,
                                   cudaMemcpyHostToDevice, s));
    CUBE_FFT(c, cufftExecR2C(c->plan_c_r2c, buf, (cufftComplex*)buf));
    k_take_imag<<<cube_grid(cspec, 256), 256, 0, s>>>((const float2*)buf, cspec, 1.0f, c->kern_c + d * cspec);
    CUBE_CUDA(c, cudaMemcpy2DAsync(bufr, pitch, raw.data() + d * n3, row, row, (size_t)nc * nc,
                                   cudaMemcpyHostToDevice, s));
    CUBE_FFT(c, cufftExecR2C(c->plan_c_r2c, bufr, (cufftComplex*)bufr));
    k_lrck<<<cube_grid(cspec, 256), 256, 0, s>>>(c->kern_c + d * cspec, (const float2*)bufr, nc, d);
  }
  // fold 1/nc^3 (a power of two: exact)
  k_scale<<<cube_grid(3 * cspec, 256), 256, 0, s>>>(c->kern_c, 3 * cspec, (float)(1.0 / ((double)nc * nc * nc)));
  CUBE_CUDA(c, cudaGetLastError());
  CUBE_CUDA(c, cudaStreamSynchronize(s));
  return CUBE_OK;
}

// ----------------------------------------------------------------- fine
int cube_fine_density_impl(cube_ctx* c, cube_stats* st, bool accumulate) {
  cudaStream_t s = c->stream;
  Geo g = make_geo(c);
  CUBE_CUDA(c, cudaMemsetAsync(c->dstats, 0, sizeof(DevStats), s));
  const int sh = dep_shift(c->p.mass_p);
  DepArgs a{g, c->xp[c->cur], c->rhoc[c->cur], c->cstart[c->cur], c->p.mass_p, c->rho_f, &c->dstats->rhof_fix, 0,
            std::ldexp(1.0f, sh), std::ldexp(1.0f, -sh), accumulate ? 1 : 0};
  cube_phase_begin(c, PH_F_DEPOSIT);
  int r = launch_fine_deposit(c, a);
  cube_phase_end(c, PH_F_DEPOSIT);
  if (r) return r;
  if (st) {
    r = cube_stats_fetch(c);
    if (r) return r;
    st->testrhof = std::ldexp((double)c->hstats->rhof_fix, -dep_shift(c->p.mass_p));
  }
  return CUBE_OK;
}

int cube_fine_forces_impl(cube_ctx* c, cube_stats* st, const float* pre) {
  int r0 = cube_fine_density_impl(c, nullptr, false);
  if (r0) return r0;
  return cube_fine_spectral_impl(c, st, pre);
}

// forces from the density on the fine mesh (pm.f90:112-126)
int cube_fine_spectral_impl(cube_ctx* c, cube_stats* st, const float* pre) {
  cudaStream_t s = c->stream;
  int64_t nfh = c->nf / 2 + 1;
  int64_t nspec = nfh * c->nf * (int64_t)c->nf;
  cube_phase_begin(c, PH_F_R2C);
  CUBE_FFT(c, cufftExecR2C(c->plan_f_r2c, c->rho_f, (cufftComplex*)c->rho_f));
  cube_phase_end(c, PH_F_R2C);
  cube_phase_begin(c, PH_F_GREEN);
  k_green3<<<cube_grid(nspec, 256), 256, 0, s>>>((const float2*)c->rho_f, c->kern_f, nspec, (float2*)c->force_f[0],
                                                  (float2*)c->force_f[1], (float2*)c->force_f[2]);
  cube_phase_end(c, PH_F_GREEN);
  cube_phase_begin(c, PH_F_C2R);
  for (int d = 0; d < 3; d++)
    CUBE_FFT(c, cufftExecC2R(c->plan_f_c2r, (cufftComplex*)c->force_f[d], c->force_f[d]));
  cube_phase_end(c, PH_F_C2R);
  cube_phase_begin(c, PH_F_F2MAX);
  if (pre)
    k_f2max<true><<<cube_grid((int64_t)c->nf * c->nf, 1, 8), 256, 0, s>>>(
        c->force_f[0], c->force_f[1], c->force_f[2], c->nf, &c->dstats->f2_fine_bits, pre[0], pre[1], c->graph_mode ? c->sd : nullptr);
  else
    k_f2max<false><<<cube_grid((int64_t)c->nf * c->nf, 1, 8), 256, 0, s>>>(
        c->force_f[0], c->force_f[1], c->force_f[2], c->nf, &c->dstats->f2_fine_bits, 0.f, 0.f, nullptr);
  cube_phase_end(c, PH_F_F2MAX);
  CUBE_CUDA(c, cudaGetLastError());
  if (st) {
    int r = cube_stats_fetch(c);
    if (r) return r;
    st->f2_max_fine = bits_float(c->hstats->f2_fine_bits);
    st->testrhof = std::ldexp((double)c->hstats->rhof_fix, -dep_shift(c->p.mass_p));
  }
  return CUBE_OK;
}

int cube_fine_kick_impl(cube_ctx* c, float a_mid, float dt, bool pre, bool with_pp) {
  KickArgs k{};
  if (with_pp) {  // the PP kick of cube_pp_launch(.., defer_kick), applied here
    if (c->graph_mode || !c->fpp) return cube_fail(c, CUBE_ERR_ARG, "PP kick in the fine kick: eager mode with PP only");
    if (c->pp_act_valid)
      k.pp_act = c->pp_act;  // the active particles are kicked; the others take the zero-kick codes here
    else
      k.fpp = c->fpp;
    k.pp_kd = (((double)a_mid * (double)dt) / 6.0) / (double)CUBE_PI_F;
    k.pp_kf = (float)k.pp_kd;
  }
  if (c->graph_mode) {  // decode with sigma_vi (slot 0), encode with sigma_vi_new (slot 1)
    cube_codec_view_dev(c, 0, &c->sd->h.cf_vi, &k.cin);
    cube_codec_view_dev(c, 1, &c->sd->cf_new, &k.cout);
    k.sd = c->sd;
  } else {
    int r = cube_codec_pair(c, c->sigma_vi, c->sigma_vi_new, &k.cin, &k.cout);
    if (r) return r;
  }
  k.g = make_geo(c);
  k.np = c->np;
  k.xp = c->xp[c->cur];
  k.vp_in = c->vp[c->cur];
  k.vp_out = c->vp[c->cur];
  k.pcell = c->pcell[c->cur];
  k.rhoc = c->rhoc[c->cur];
  k.cstart = c->cstart[c->cur];
  k.vfield = c->vfield[c->cur];
  for (int d = 0; d < 3; d++) k.f[d] = c->force_f[d];
  k.a_mid = a_mid;
  k.dt = dt;
  k.vmax_bits = nullptr;
  k.nexact = &c->dstats->nexact;
  k.exact_only = c->opt_exact_kicks;
  // after an upload or initial conditions the last vmax is unknown: the fine
  // kick then records the velocities' maxima for the coarse kick's threshold
  // (the fine density of this step zeroed the estimate)
  if (!c->graph_mode && c->vmax_prev[0] == 0.f && c->vmax_prev[1] == 0.f && c->vmax_prev[2] == 0.f)
    k.vmax_est = c->dstats->vmax_est_bits;
  cube_phase_begin(c, PH_F_KICK);
  if (pre)
    k_kick<true, true><<<cube_grid(c->np, 256), 256, 0, c->stream>>>(k);
  else
    k_kick<true, false><<<cube_grid(c->np, 256), 256, 0, c->stream>>>(k);
  cube_phase_end(c, PH_F_KICK);
  CUBE_CUDA(c, cudaGetLastError());
  return CUBE_OK;
}

// CIC density of the particles on an ng^3 mesh (ng = nc, 2 nc or 4 nc) for the
// power spectrum, mass 1 per particle (cicpower.f90:79,100-133), into the
// padded mesh rho; *total receives the exact fixed-point sum.
int cube_pk_deposit(cube_ctx* c, int ng, float* rho, unsigned long long* total) {
  const int sh = dep_shift(1.0f);
  DepArgs a{make_geo(c), c->xp[c->cur], c->rhoc[c->cur], c->cstart[c->cur], 1.0f, rho, total, ng,
            std::ldexp(1.0f, sh), std::ldexp(1.0f, -sh), 0};
  int nc = c->p.nc;
  if (ng == nc) return launch_deposit<1, 8, 8, 8, 1, 1, true>(c, a);
  if (ng == 2 * nc) return launch_deposit<2, 8, 8, 4, 1, 1, true>(c, a);
  if (ng == 4 * nc) return launch_deposit<4, 8, 4, 4, 1, 1, true>(c, a);
  return cube_fail(c, CUBE_ERR_ARG, "power-spectrum mesh must be nc, 2nc or 4nc per dimension");
}

// --------------------------------------------------------------- coarse
int cube_coarse_density_impl(cube_ctx* c, cube_stats* st, bool accumulate) {
  Geo g = make_geo(c);
  CUBE_CUDA(c, cudaMemsetAsync(&c->dstats->f2_coarse_bits, 0, 4, c->stream));
  CUBE_CUDA(c, cudaMemsetAsync(&c->dstats->rhoc_fix, 0, 8, c->stream));
  const int sh = dep_shift(c->p.mass_p);
  DepArgs a{g, c->xp[c->cur], c->rhoc[c->cur], c->cstart[c->cur], c->p.mass_p, c->rho_c, &c->dstats->rhoc_fix, 0,
            std::ldexp(1.0f, sh), std::ldexp(1.0f, -sh), accumulate ? 1 : 0};
  cube_phase_begin(c, PH_C_DEPOSIT);
  int r = launch_coarse_deposit(c, a);
  cube_phase_end(c, PH_C_DEPOSIT);
  if (r) return r;
  if (st) {
    r = cube_stats_fetch(c);
    if (r) return r;
    st->testrhoc = std::ldexp((double)c->hstats->rhoc_fix, -dep_shift(c->p.mass_p));
  }
  return CUBE_OK;
}

int cube_coarse_forces_impl(cube_ctx* c, cube_stats* st, const float* pre) {
  int r0 = cube_coarse_density_impl(c, nullptr, false);
  if (r0) return r0;
  return cube_coarse_spectral_impl(c, st, pre);
}

// forces from the density on the coarse mesh (pm.f90:275-315)
int cube_coarse_spectral_impl(cube_ctx* c, cube_stats* st, const float* pre) {
  cudaStream_t s = c->stream;
  int nc = c->p.nc;
  int64_t nch = nc / 2 + 1;
  int64_t cspec = nch * nc * (int64_t)nc;
  cube_phase_begin(c, PH_C_FFT);
  CUBE_FFT(c, cufftExecR2C(c->plan_c_r2c, c->rho_c, (cufftComplex*)c->rho_c));
  k_green3<<<cube_grid(cspec, 256), 256, 0, s>>>((const float2*)c->rho_c, c->kern_c, cspec, (float2*)c->force_c[0],
                                                  (float2*)c->force_c[1], (float2*)c->force_c[2]);
  for (int d = 0; d < 3; d++)
    CUBE_FFT(c, cufftExecC2R(c->plan_c_c2r, (cufftComplex*)c->force_c[d], c->force_c[d]));
  if (pre)
    k_f2max<true><<<cube_grid((int64_t)nc * nc, 1, 8), 256, 0, s>>>(c->force_c[0], c->force_c[1], c->force_c[2], nc,
                                                                    &c->dstats->f2_coarse_bits, pre[0], pre[1], c->graph_mode ? c->sd : nullptr);
  else
    k_f2max<false><<<cube_grid((int64_t)nc * nc, 1, 8), 256, 0, s>>>(c->force_c[0], c->force_c[1], c->force_c[2], nc,
                                                                     &c->dstats->f2_coarse_bits, 0.f, 0.f, nullptr);
  cube_phase_end(c, PH_C_FFT);
  CUBE_CUDA(c, cudaGetLastError());
  if (st) {
    int r = cube_stats_fetch(c);
    if (r) return r;
    st->f2_max_coarse = bits_float(c->hstats->f2_coarse_bits);
    st->testrhoc = std::ldexp((double)c->hstats->rhoc_fix, -dep_shift(c->p.mass_p));
  }
  return CUBE_OK;
}

int cube_coarse_kick_impl(cube_ctx* c, float a_mid, float dt, cube_stats* st, bool pre) {
  KickArgs k{};
  int r;
  if (c->graph_mode) {  // sigma_vi is now sigma_vi_new (slot 1) for both
    cube_codec_view_dev(c, 1, &c->sd->cf_new, &k.cin);
    cube_codec_view_dev(c, 1, &c->sd->cf_new, &k.cout);
    k.sd = c->sd;
  } else {
    r = cube_codec_pair(c, c->sigma_vi, c->sigma_vi, &k.cin, &k.cout);
    if (r) return r;
  }
  int cur = c->cur, alt = 1 - cur;
  CUBE_CUDA(c, cudaMemsetAsync(c->dstats->vmax_bits, 0, 12, c->stream));
  CUBE_CUDA(c, cudaMemsetAsync(c->dstats->vmax_lo_bits, 0, 12, c->stream));
  CUBE_CUDA(c, cudaMemsetAsync(&c->dstats->nexact, 0, 8, c->stream));
  k.g = make_geo(c);
  k.np = c->np;
  k.xp = c->xp[cur];
  k.vp_in = c->vp[cur];
  k.vp_out = c->vp[alt];  // the input codes stay intact for an exact vmax rerun
  k.pcell = c->pcell[cur];
  k.vfield = c->vfield[cur];
  for (int d = 0; d < 3; d++) {
    k.f[d] = c->force_c[d];
    // velocities change little per step: every lane that could reach 0.95 of
    // the last vmax is evaluated exactly; if the maximum ends below that, a
    // rerun evaluates the lanes that could reach this pass's largest lower
    // bound (the maximum's lane among them)
    k.tau[d] = kVmaxTau * c->vmax_prev[d];
  }
  // last vmax unknown: 0.7 of the fine kick's FP32 maxima instead (zero when
  // no fine kick recorded them: every lane exact)
  const bool est = !c->graph_mode && c->vmax_prev[0] == 0.f && c->vmax_prev[1] == 0.f && c->vmax_prev[2] == 0.f;
  if (est) k.tau_est = c->dstats->vmax_est_bits;
  k.a_mid = a_mid;
  k.dt = dt;
  k.vmax_bits = c->dstats->vmax_bits;
  k.vmax_lo = c->dstats->vmax_lo_bits;
  k.nexact = &c->dstats->nexact;
  k.vmax_only = 0;
  k.exact_only = c->opt_exact_kicks;
  cube_phase_begin(c, PH_C_KICK);
  if (c->vp_host && !c->graph_mode) {
    // a download is waiting for vp: kick in eight pieces of particles, each
    // piece's codes going to the host while the next is kicked
    const size_t bx = 3 * (size_t)c->p.izipx, bv = 3 * (size_t)c->p.izipv;
    for (int i = 0; i < 8; i++) {
      const int64_t p0 = c->np * i / 8, p1 = c->np * (i + 1) / 8;
      if (p1 <= p0) continue;
      KickArgs kp = k;
      kp.np = p1 - p0;
      kp.xp = (const char*)k.xp + bx * p0;
      kp.vp_in = (const char*)k.vp_in + bv * p0;
      kp.vp_out = (char*)k.vp_out + bv * p0;
      kp.pcell = k.pcell + p0;
      if (pre)
        k_kick<false, true><<<cube_grid(kp.np, 256), 256, 0, c->stream>>>(kp);
      else
        k_kick<false, false><<<cube_grid(kp.np, 256), 256, 0, c->stream>>>(kp);
      CUBE_CUDA(c, cudaEventRecord(c->ev_copy_start, c->stream));
      CUBE_CUDA(c, cudaStreamWaitEvent(c->stream_copy, c->ev_copy_start, 0));
      CUBE_CUDA(c, cudaMemcpyAsync((char*)c->vp_host + bv * p0, kp.vp_out, bv * (p1 - p0), cudaMemcpyDeviceToHost,
                                   c->stream_copy));
    }
    CUBE_CUDA(c, cudaEventRecord(c->ev_copy, c->stream_copy));
    c->copy_pending = true;
    c->vp_host = nullptr;
  } else if (pre)
    k_kick<false, true><<<cube_grid(c->np, 256), 256, 0, c->stream>>>(k);
  else
    k_kick<false, false><<<cube_grid(c->np, 256), 256, 0, c->stream>>>(k);
  cube_phase_end(c, PH_C_KICK);
  CUBE_CUDA(c, cudaGetLastError());
  if (c->graph_mode) {
    // the exact rerun decides on the device whether it runs; the stats of the
    // whole particle_mesh go to the host's copy
    k.vmax_only = 1;
    if (pre)
      k_kick<false, true><<<cube_grid(c->np, 256), 256, 0, c->stream>>>(k);
    else
      k_kick<false, false><<<cube_grid(c->np, 256), 256, 0, c->stream>>>(k);
    CUBE_CUDA(c, cudaGetLastError());
    CUBE_CUDA(c, cudaMemcpyAsync(&c->sout->coarse, c->dstats, sizeof(DevStats), cudaMemcpyDeviceToDevice, c->stream));
    void* t = c->vp[cur];
    c->vp[cur] = c->vp[alt];
    c->vp[alt] = t;
    return CUBE_OK;
  }
  r = cube_stats_fetch(c);
  if (r) return r;
  float vm[3];
  bool rerun = false;
  for (int d = 0; d < 3; d++) {
    vm[d] = bits_float(c->hstats->vmax_bits[d]);
    const float tau = est ? 0.7f * bits_float(c->hstats->vmax_est_bits[d]) : k.tau[d];
    if (!(vm[d] >= tau)) rerun = true;
  }
  unsigned long long nex = c->hstats->nexact;
  if (rerun) {
    CUBE_CUDA(c, cudaMemsetAsync(c->dstats->vmax_bits, 0, 12, c->stream));
    k.vmax_only = 1;
    if (pre)
      k_kick<false, true><<<cube_grid(c->np, 256), 256, 0, c->stream>>>(k);
    else
      k_kick<false, false><<<cube_grid(c->np, 256), 256, 0, c->stream>>>(k);
    CUBE_CUDA(c, cudaGetLastError());
    r = cube_stats_fetch(c);
    if (r) return r;
    for (int d = 0; d < 3; d++) vm[d] = bits_float(c->hstats->vmax_bits[d]);
  }
  void* t = c->vp[cur];
  c->vp[cur] = c->vp[alt];
  c->vp[alt] = t;
  for (int d = 0; d < 3; d++) c->vmax_prev[d] = vm[d];
  c->kick_exact_lanes = nex;
  if (st) {
    for (int d = 0; d < 3; d++) st->vmax[d] = vm[d];
    st->f2_max_coarse = bits_float(c->hstats->f2_coarse_bits);
    st->testrhoc = std::ldexp((double)c->hstats->rhoc_fix, -dep_shift(c->p.mass_p));
  }
  return CUBE_OK;
}
