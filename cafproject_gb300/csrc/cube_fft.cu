// cube_fft.cu -- the fine mesh's force chain (pm.f90:112-126) as this
// library's own transforms, for power-of-two meshes of 64 to 2048 points a
// side; other sizes keep cuFFT (cube_pm.cu).
//
// The reference transforms the density once (R2C), multiplies by i*K_d for
// each force component and transforms each product back (C2R), then takes
// the maximum of |F|^2 (pm.f90:113-126).  With cuFFT those are six passes
// over the 1024^3 mesh per component plus a multiply pass and a maxima pass.
// Here the same arithmetic runs in five passes, each a set of
// one-dimensional FFTs done in shared memory:
//   1. rows (x): two real rows as one complex FFT, split into the two
//      half spectra, in place (R2C along x);
//   2. columns along y, in place;
//   3. columns along z, then, with the spectrum still in shared memory, for
//      each d: multiply by i*K_d and transform back along z into force_f[d]
//      (the Green's multiply and the first inverse pass fused);
//   4. columns along y of the three force meshes, inverse, in place;
//   5. rows: each pair of half-spectrum rows of each component back to two
//      real rows (C2R along x), then |F|^2 of every point (maxval of
//      pm.f90:126, in the reference's order (fx^2+fy^2)+fz^2) and, in the
//      fused step, each value rewritten as its kick factor.
// The one-dimensional transforms are Stockham radix-16/8/4/2 stages on
// shared memory with twiddles W_N^m tabulated once from double precision; the
// inverse is the forward transform of the conjugate, conjugated.  Like
// cuFFT, neither direction normalises (the kernel K carries 1/nf^3).
#include <algorithm>
#include <cmath>
#include <vector>

#include "cube_internal.cuh"

namespace {

// ------------------------------------------------------------ complex math
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(__fmaf_rn(a.x, b.x, -a.y * b.y), __fmaf_rn(a.x, b.y, a.y * b.x));
}
__device__ __forceinline__ float2 mul_mi(float2 a) { return make_float2(a.y, -a.x); }  // a * (-i)
__device__ __forceinline__ float2 conjf2(float2 a) { return make_float2(a.x, -a.y); }

// in-register DFTs (forward, exp(-2 pi i jk/R)) of R = 2, 4, 8, 16 points
__device__ __forceinline__ void dft2(float2& a, float2& b) {
  const float2 t = a;
  a = cadd(t, b);
  b = csub(t, b);
}
__device__ __forceinline__ void dft4(float2& x0, float2& x1, float2& x2, float2& x3) {
  const float2 a = cadd(x0, x2), b = csub(x0, x2), c = cadd(x1, x3), d = mul_mi(csub(x1, x3));
  x0 = cadd(a, c);
  x2 = csub(a, c);
  x1 = cadd(b, d);
  x3 = csub(b, d);
}
constexpr float kS2 = 0.70710678118654752f;  // cos(pi/4)
template <int R>
__device__ __forceinline__ void dft(float2* v);
template <>
__device__ __forceinline__ void dft<2>(float2* v) {
  dft2(v[0], v[1]);
}
template <>
__device__ __forceinline__ void dft<4>(float2* v) {
  dft4(v[0], v[1], v[2], v[3]);
}
// 8 = 4 x 2: n = 2 n1 + n2, k = k1 + 4 k2
template <>
__device__ __forceinline__ void dft<8>(float2* v) {
  float2 a[2][4];
#pragma unroll
  for (int n2 = 0; n2 < 2; n2++) {
#pragma unroll
    for (int n1 = 0; n1 < 4; n1++) a[n2][n1] = v[2 * n1 + n2];
    dft4(a[n2][0], a[n2][1], a[n2][2], a[n2][3]);
  }
  // W8^{k1} on n2 = 1
  a[1][1] = make_float2(kS2 * (a[1][1].x + a[1][1].y), kS2 * (a[1][1].y - a[1][1].x));
  a[1][2] = mul_mi(a[1][2]);
  a[1][3] = make_float2(kS2 * (a[1][3].y - a[1][3].x), -kS2 * (a[1][3].x + a[1][3].y));
#pragma unroll
  for (int k1 = 0; k1 < 4; k1++) {
    float2 p = a[0][k1], q = a[1][k1];
    dft2(p, q);
    v[k1] = p;
    v[k1 + 4] = q;
  }
}
// 16 = 4 x 4: n = 4 n1 + n2, k = k1 + 4 k2
__constant__ float2 c_w16[10] = {
    {1.0f, 0.0f},
    {0.92387953251128674f, -0.38268343236508977f},
    {0.70710678118654752f, -0.70710678118654752f},
    {0.38268343236508977f, -0.92387953251128674f},
    {0.0f, -1.0f},
    {-0.38268343236508977f, -0.92387953251128674f},
    {-0.70710678118654752f, -0.70710678118654752f},
    {-0.92387953251128674f, -0.38268343236508977f},
    {-1.0f, 0.0f},
    {-0.92387953251128674f, 0.38268343236508977f}};
template <>
__device__ __forceinline__ void dft<16>(float2* v) {
  float2 a[4][4];
#pragma unroll
  for (int n2 = 0; n2 < 4; n2++) {
#pragma unroll
    for (int n1 = 0; n1 < 4; n1++) a[n2][n1] = v[4 * n1 + n2];
    dft4(a[n2][0], a[n2][1], a[n2][2], a[n2][3]);
  }
#pragma unroll
  for (int n2 = 1; n2 < 4; n2++)
#pragma unroll
    for (int k1 = 1; k1 < 4; k1++) a[n2][k1] = cmul(a[n2][k1], c_w16[n2 * k1]);
#pragma unroll
  for (int k1 = 0; k1 < 4; k1++) {
    float2 p = a[0][k1], q = a[1][k1], r = a[2][k1], s = a[3][k1];
    dft4(p, q, r, s);
    v[k1] = p;
    v[k1 + 4] = q;
    v[k1 + 8] = r;
    v[k1 + 12] = s;
  }
}

// radix of stage s of an N-point transform: 16s first, then the remainder
template <int N, int S>
struct Radix {
  static constexpr int span = Radix<N, S - 1>::span * Radix<N, S - 1>::r;  // Ns before this stage
  static constexpr int rem = N / span;
  static constexpr int r = rem >= 16 ? 16 : rem;
};
template <int N>
struct Radix<N, 0> {
  static constexpr int span = 1;
  static constexpr int r = N >= 16 ? 16 : N;
};
template <int N>
constexpr int nstages() {
  int s = 0, m = N;
  while (m > 1) {
    m /= m >= 16 ? 16 : m;
    s++;
  }
  return s;
}

// Shared-memory index of element i of line l.  Column passes interleave
// their L lines (a global row of L consecutive columns lands contiguously);
// row passes store each line contiguously.  One padding element every 16
// elements spreads the stride-16 accesses of the radix-16 stages over the
// banks.
template <int N, int L, bool kRows>
__device__ __forceinline__ int sidx(int i, int l) {
  return kRows ? l * (N + N / 16) + i + (i >> 4) : (i + (i >> 4)) * L + l;
}
template <int N, int L>
constexpr int smem_elems() {
  return (N + N / 16) * L;
}

// One Stockham stage of an N-point forward transform of L lines held in
// shared memory (in place: every thread reads its inputs, a barrier, then
// the writes).  Items (l, j), j < N/R, are spread over the block's 256
// threads, consecutive threads on consecutive j (rows) or l (columns).
template <int N, int L, bool kRows, int S>
__device__ __forceinline__ void stockham_stage(float2* s, const float2* __restrict__ tw) {
  constexpr int R = Radix<N, S>::r, Ns = Radix<N, S>::span, NJ = N / R, ITEMS = NJ * L;
  constexpr int PER = (ITEMS + 255) / 256;
  float2 v[PER][R];
#pragma unroll
  for (int q = 0; q < PER; q++) {
    const int it = threadIdx.x + 256 * q;
    if (ITEMS % 256 == 0 || it < ITEMS) {
      const int l = kRows ? it / NJ : it % L, j = kRows ? it % NJ : it / L, k = j & (Ns - 1);
#pragma unroll
      for (int r = 0; r < R; r++) {
        float2 x = s[sidx<N, L, kRows>(j + r * NJ, l)];
        if (Ns > 1 && r > 0) x = cmul(x, __ldg(tw + (k * r * (N / (Ns * R)))));
        v[q][r] = x;
      }
      dft<R>(v[q]);
    }
  }
  __syncthreads();
#pragma unroll
  for (int q = 0; q < PER; q++) {
    const int it = threadIdx.x + 256 * q;
    if (ITEMS % 256 == 0 || it < ITEMS) {
      const int l = kRows ? it / NJ : it % L, j = kRows ? it % NJ : it / L, k = j & (Ns - 1);
      const int base = (j / Ns) * Ns * R + k;
#pragma unroll
      for (int r = 0; r < R; r++) s[sidx<N, L, kRows>(base + r * Ns, l)] = v[q][r];
    }
  }
  __syncthreads();
}

// the stages S = 0 .. nstages<N>()-1 in order
template <int N, int L, bool kRows, int S, bool kDone = (S >= nstages<N>())>
struct StageLoop;
template <int N, int L, bool kRows, int S>
struct StageLoop<N, L, kRows, S, false> {
  __device__ __forceinline__ static void run(float2* s, const float2* tw) {
    stockham_stage<N, L, kRows, S>(s, tw);
    StageLoop<N, L, kRows, S + 1>::run(s, tw);
  }
};
template <int N, int L, bool kRows, int S>
struct StageLoop<N, L, kRows, S, true> {
  __device__ __forceinline__ static void run(float2*, const float2*) {}
};
// forward transform of the L lines in s (ends with a barrier)
template <int N, int L, bool kRows>
__device__ __forceinline__ void fft_lines(float2* s, const float2* tw) {
  StageLoop<N, L, kRows, 0>::run(s, tw);
}

// lines per block: at most 32 complex values per thread in a stage
constexpr int lines_for(int n, int cap) { return 8192 / n < cap ? 8192 / n : cap; }

// ------------------------------------------------------------------ passes
// Every pass runs 256 threads per block.

// The inverse transforms are the forward transform of the conjugate, conjugated
// (unnormalised, as cuFFT's).

// Pass 1: R2C along x.  Each block takes 2L real rows, packs row pairs as
// z = a + i b, transforms, and splits A[k] = (Z[k] + conj Z[N-k])/2,
// B[k] = (Z[k] - conj Z[N-k])/(2i), k = 0..N/2, written in place.
template <int N, int L>
__global__ void __launch_bounds__(256) k_fft_x_r2c(float* __restrict__ mesh, int64_t nrows,
                                                   const float2* __restrict__ tw) {
  extern __shared__ float2 sm[];
  const int64_t row0 = (int64_t)blockIdx.x * 2 * L;
  const int pitch = N + 2;
  for (int i = threadIdx.x; i < N * L; i += 256) {
    const int l = i / N, x = i % N;
    const int64_t ra = row0 + 2 * l, rb = ra + 1;
    const float a = ra < nrows ? mesh[ra * pitch + x] : 0.f;
    const float b = rb < nrows ? mesh[rb * pitch + x] : 0.f;
    sm[sidx<N, L, true>(x, l)] = make_float2(a, b);
  }
  __syncthreads();
  fft_lines<N, L, true>(sm, tw);
  for (int i = threadIdx.x; i < (N / 2 + 1) * L; i += 256) {
    const int l = i / (N / 2 + 1), k = i % (N / 2 + 1);
    const float2 z = sm[sidx<N, L, true>(k, l)], w = conjf2(sm[sidx<N, L, true>((N - k) & (N - 1), l)]);
    const float2 A = make_float2(0.5f * (z.x + w.x), 0.5f * (z.y + w.y));
    const float2 B = make_float2(0.5f * (z.y - w.y), -0.5f * (z.x - w.x));  // (z - w) / (2i)
    const int64_t ra = row0 + 2 * l, rb = ra + 1;
    if (ra < nrows) reinterpret_cast<float2*>(mesh + ra * pitch)[k] = A;
    if (rb < nrows) reinterpret_cast<float2*>(mesh + rb * pitch)[k] = B;
  }
}

// Pass 2 / 4: transforms along y of the half spectrum, in place.  Block:
// plane z (blockIdx.y), columns kx0 .. kx0+L-1 (blockIdx.x), mesh
// blockIdx.z of the three (pass 4) or the density (pass 2).
template <int N, int L, bool kInv>
__global__ void __launch_bounds__(256) k_fft_y(float2* m0, float2* m1, float2* m2, const float2* __restrict__ tw) {
  extern __shared__ float2 sm[];
  constexpr int P = N / 2 + 1;
  float2* m = blockIdx.z == 0 ? m0 : (blockIdx.z == 1 ? m1 : m2);
  const int kx0 = blockIdx.x * L;
  const int64_t zoff = (int64_t)blockIdx.y * N * P;
  for (int i = threadIdx.x; i < N * L; i += 256) {
    const int l = i % L, y = i / L, kx = kx0 + l;
    float2 v = kx < P ? m[zoff + (int64_t)y * P + kx] : make_float2(0.f, 0.f);
    if (kInv) v.y = -v.y;
    sm[sidx<N, L, false>(y, l)] = v;
  }
  __syncthreads();
  fft_lines<N, L, false>(sm, tw);
  for (int i = threadIdx.x; i < N * L; i += 256) {
    const int l = i % L, y = i / L, kx = kx0 + l;
    float2 v = sm[sidx<N, L, false>(y, l)];
    if (kInv) v.y = -v.y;
    if (kx < P) m[zoff + (int64_t)y * P + kx] = v;
  }
}

// Pass 3: transforms along z, the Green's multiply and the inverse along z
// (pm.f90:117-121: re = -Im(rho)*K_d, im = Re(rho)*K_d).  Block: row ky
// (blockIdx.y), columns kx0 .. kx0+L-1.  The spectrum stays in buffer A; each
// component is formed in buffer B, transformed back and stored.
template <int N, int L>
__global__ void __launch_bounds__(256) k_fft_z_green(const float2* __restrict__ rho, const float* __restrict__ kern,
                                                     float2* f0, float2* f1, float2* f2,
                                                     const float2* __restrict__ tw) {
  extern __shared__ float2 sm[];
  constexpr int P = N / 2 + 1;
  constexpr int64_t NS = (int64_t)P * N * N;
  float2* A = sm;
  float2* B = sm + smem_elems<N, L>();
  const int kx0 = blockIdx.x * L, ky = blockIdx.y;
  for (int i = threadIdx.x; i < N * L; i += 256) {
    const int l = i % L, z = i / L, kx = kx0 + l;
    A[sidx<N, L, false>(z, l)] = kx < P ? rho[((int64_t)z * N + ky) * P + kx] : make_float2(0.f, 0.f);
  }
  __syncthreads();
  fft_lines<N, L, false>(A, tw);
  for (int d = 0; d < 3; d++) {
    const float* K = kern + d * NS;
    for (int i = threadIdx.x; i < N * L; i += 256) {
      const int l = i % L, z = i / L, kx = kx0 + l;
      const float k = kx < P ? __ldg(K + ((int64_t)z * N + ky) * P + kx) : 0.f;
      const float2 a = A[sidx<N, L, false>(z, l)];
      // i*K*a, conjugated for the inverse transform
      B[sidx<N, L, false>(z, l)] = make_float2(-a.y * k, -(a.x * k));
    }
    __syncthreads();
    fft_lines<N, L, false>(B, tw);
    float2* f = d == 0 ? f0 : (d == 1 ? f1 : f2);
    for (int i = threadIdx.x; i < N * L; i += 256) {
      const int l = i % L, z = i / L, kx = kx0 + l;
      const float2 v = B[sidx<N, L, false>(z, l)];
      if (kx < P) f[((int64_t)z * N + ky) * P + kx] = make_float2(v.x, -v.y);
    }
    __syncthreads();
  }
}

// Pass 5: C2R along x of the three components, |F|^2 and the kick factors.
// Block: 2L rows; per component, row pairs (a, b) with half spectra Xa, Xb
// become Z[k] = Xa[k] + i Xb[k] over the full length (Xa[N-k] = conj Xa[k]),
// whose inverse transform is a + i b.  The half spectra's k = 0 and N/2
// terms are taken real, as the C2R of a real field.
template <int N, int L, bool kPre>
__global__ void __launch_bounds__(256) k_fft_x_c2r_f2(float* f0, float* f1, float* f2, int64_t nrows,
                                                      const float2* __restrict__ tw, unsigned int* __restrict__ f2max,
                                                      float a_mid, float dt, const StepDev* sd) {
  extern __shared__ float2 sm[];
  __shared__ float wmax[8];
  if (kPre && sd) {
    a_mid = sd->h.a_mid;
    dt = sd->h.dt;
  }
  const int pitch = N + 2;
  constexpr int H = N / 2;
  float m = 0.f;
  for (int64_t row0 = (int64_t)blockIdx.x * 2 * L; row0 < nrows; row0 += (int64_t)gridDim.x * 2 * L) {
    for (int d = 0; d < 3; d++) {
      const float* f = d == 0 ? f0 : (d == 1 ? f1 : f2);
      float2* S = sm + d * smem_elems<N, L>();
      for (int i = threadIdx.x; i < N * L; i += 256) {
        const int l = i / N, k = i % N;
        const int64_t ra = row0 + 2 * l, rb = ra + 1;
        const int kk = k <= H ? k : N - k;
        float2 xa = ra < nrows ? reinterpret_cast<const float2*>(f + ra * pitch)[kk] : make_float2(0.f, 0.f);
        float2 xb = rb < nrows ? reinterpret_cast<const float2*>(f + rb * pitch)[kk] : make_float2(0.f, 0.f);
        if (kk == 0 || kk == H) xa.y = xb.y = 0.f;
        if (k > H) {
          xa.y = -xa.y;
          xb.y = -xb.y;
        }
        // Z = Xa + i Xb, conjugated for the inverse transform
        S[sidx<N, L, true>(k, l)] = make_float2(xa.x - xb.y, -(xa.y + xb.x));
      }
    }
    __syncthreads();
    for (int d = 0; d < 3; d++) fft_lines<N, L, true>(sm + d * smem_elems<N, L>(), tw);
    // z = conj(result) = a + i b: a = x, b = -y
    for (int i = threadIdx.x; i < N * L; i += 256) {
      const int l = i / N, x = i % N;
      const int64_t ra = row0 + 2 * l, rb = ra + 1;
      const float2 u = sm[sidx<N, L, true>(x, l)], v = sm[smem_elems<N, L>() + sidx<N, L, true>(x, l)],
                   w = sm[2 * smem_elems<N, L>() + sidx<N, L, true>(x, l)];
      const float ax = u.x, ay = v.x, az = w.x, bx = -u.y, by = -v.y, bz = -w.y;
      if (ra < nrows) {
        m = fmaxf(m, __fadd_rn(__fadd_rn(__fmul_rn(ax, ax), __fmul_rn(ay, ay)), __fmul_rn(az, az)));
        f0[ra * pitch + x] = kPre ? kick_pre(ax, a_mid, dt) : ax;
        f1[ra * pitch + x] = kPre ? kick_pre(ay, a_mid, dt) : ay;
        f2[ra * pitch + x] = kPre ? kick_pre(az, a_mid, dt) : az;
      }
      if (rb < nrows) {
        m = fmaxf(m, __fadd_rn(__fadd_rn(__fmul_rn(bx, bx), __fmul_rn(by, by)), __fmul_rn(bz, bz)));
        f0[rb * pitch + x] = kPre ? kick_pre(bx, a_mid, dt) : bx;
        f1[rb * pitch + x] = kPre ? kick_pre(by, a_mid, dt) : by;
        f2[rb * pitch + x] = kPre ? kick_pre(bz, a_mid, dt) : bz;
      }
    }
    __syncthreads();
  }
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) wmax[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < 8; w++) m = fmaxf(m, wmax[w]);
    atomic_max_pos(f2max, m);
  }
}

// lines per block of each pass (row pairs for the x passes)
template <int N>
struct Lines {
  static constexpr int x = lines_for(N, 4), y = lines_for(N, 8), z = lines_for(N, 4),
                       c2r = lines_for(N, 4) / 2 > 0 ? lines_for(N, 4) / 2 : 1;
};

template <int N>
int run_chain(cube_ctx* c, const float* pre) {
  using Ln = Lines<N>;
  cudaStream_t s = c->stream;
  const int64_t nrows = (int64_t)N * N;
  constexpr int P = N / 2 + 1;
  const float2* tw = c->fft_tw;
  float2* rho = reinterpret_cast<float2*>(c->rho_f);
  float2* f[3] = {reinterpret_cast<float2*>(c->force_f[0]), reinterpret_cast<float2*>(c->force_f[1]),
                  reinterpret_cast<float2*>(c->force_f[2])};
  const size_t sx = sizeof(float2) * smem_elems<N, Ln::x>(), sy = sizeof(float2) * smem_elems<N, Ln::y>(),
               sz = 2 * sizeof(float2) * smem_elems<N, Ln::z>(), s5 = 3 * sizeof(float2) * smem_elems<N, Ln::c2r>();
  cube_phase_begin(c, PH_F_R2C);
  k_fft_x_r2c<N, Ln::x><<<(unsigned)((nrows + 2 * Ln::x - 1) / (2 * Ln::x)), 256, sx, s>>>(c->rho_f, nrows, tw);
  k_fft_y<N, Ln::y, false><<<dim3((P + Ln::y - 1) / Ln::y, N, 1), 256, sy, s>>>(rho, rho, rho, tw);
  cube_phase_end(c, PH_F_R2C);
  cube_phase_begin(c, PH_F_GREEN);
  k_fft_z_green<N, Ln::z><<<dim3((P + Ln::z - 1) / Ln::z, N, 1), 256, sz, s>>>(rho, c->kern_f, f[0], f[1], f[2], tw);
  cube_phase_end(c, PH_F_GREEN);
  cube_phase_begin(c, PH_F_C2R);
  k_fft_y<N, Ln::y, true><<<dim3((P + Ln::y - 1) / Ln::y, N, 3), 256, sy, s>>>(f[0], f[1], f[2], tw);
  cube_phase_end(c, PH_F_C2R);
  cube_phase_begin(c, PH_F_F2MAX);
  const int64_t groups = (nrows + 2 * Ln::c2r - 1) / (2 * Ln::c2r);
  const unsigned nb5 = (unsigned)std::min<int64_t>(groups, cube_grid(groups, 1, 4));
  if (pre)
    k_fft_x_c2r_f2<N, Ln::c2r, true><<<nb5, 256, s5, s>>>(c->force_f[0], c->force_f[1], c->force_f[2], nrows, tw,
                                                           &c->dstats->f2_fine_bits, pre[0], pre[1],
                                                           c->graph_mode ? c->sd : nullptr);
  else
    k_fft_x_c2r_f2<N, Ln::c2r, false><<<nb5, 256, s5, s>>>(c->force_f[0], c->force_f[1], c->force_f[2], nrows, tw,
                                                            &c->dstats->f2_fine_bits, 0.f, 0.f, nullptr);
  cube_phase_end(c, PH_F_F2MAX);
  CUBE_CUDA(c, cudaGetLastError());
  return CUBE_OK;
}

template <int N>
int set_attrs(cube_ctx* c) {
  using Ln = Lines<N>;
  const int sx = (int)(sizeof(float2) * smem_elems<N, Ln::x>()), sy = (int)(sizeof(float2) * smem_elems<N, Ln::y>()),
            sz = (int)(2 * sizeof(float2) * smem_elems<N, Ln::z>()),
            s5 = (int)(3 * sizeof(float2) * smem_elems<N, Ln::c2r>());
  CUBE_CUDA(c, cudaFuncSetAttribute(k_fft_x_r2c<N, Ln::x>, cudaFuncAttributeMaxDynamicSharedMemorySize, sx));
  CUBE_CUDA(c, cudaFuncSetAttribute(k_fft_y<N, Ln::y, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, sy));
  CUBE_CUDA(c, cudaFuncSetAttribute(k_fft_y<N, Ln::y, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, sy));
  CUBE_CUDA(c, cudaFuncSetAttribute(k_fft_z_green<N, Ln::z>, cudaFuncAttributeMaxDynamicSharedMemorySize, sz));
  CUBE_CUDA(c, cudaFuncSetAttribute(k_fft_x_c2r_f2<N, Ln::c2r, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, s5));
  CUBE_CUDA(c, cudaFuncSetAttribute(k_fft_x_c2r_f2<N, Ln::c2r, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    s5));
  return CUBE_OK;
}

}  // namespace

// Twiddles W_N^m = exp(-2 pi i m/N), m < N, from double precision, and the
// kernels' shared-memory sizes; the context then takes this path for its
// fine mesh when nf is a power of two in [64, 2048].
int cube_fft_init(cube_ctx* c) {
  const int n = c->nf;
  c->fft_own = false;
  if (n < 64 || n > 2048 || (n & (n - 1))) return CUBE_OK;
  std::vector<float2> w(n);
  for (int m = 0; m < n; m++) {
    const double a = -2.0 * 3.14159265358979323846 * (double)m / (double)n;
    w[m] = make_float2((float)std::cos(a), (float)std::sin(a));
  }
  CUBE_CUDA(c, cudaMalloc(&c->fft_tw, sizeof(float2) * n));
  CUBE_CUDA(c, cudaMemcpy(c->fft_tw, w.data(), sizeof(float2) * n, cudaMemcpyHostToDevice));
  int r;
  switch (n) {
    case 64: r = set_attrs<64>(c); break;
    case 128: r = set_attrs<128>(c); break;
    case 256: r = set_attrs<256>(c); break;
    case 512: r = set_attrs<512>(c); break;
    case 1024: r = set_attrs<1024>(c); break;
    default: r = set_attrs<2048>(c); break;
  }
  if (r) return r;
  c->fft_own = true;
  return CUBE_OK;
}

// The force chain of pm.f90:112-126 on the fine mesh whose density is in
// rho_f: spectrum, i*K_d, back to the three force meshes, |F|^2 maxima into
// dstats, and with pre (a_mid, dt) the kick factors.  The density buffer
// then holds the spectrum, as after cuFFT's in-place R2C.
int cube_fine_chain_own(cube_ctx* c, const float* pre) {
  switch (c->nf) {
    case 64: return run_chain<64>(c, pre);
    case 128: return run_chain<128>(c, pre);
    case 256: return run_chain<256>(c, pre);
    case 512: return run_chain<512>(c, pre);
    case 1024: return run_chain<1024>(c, pre);
    case 2048: return run_chain<2048>(c, pre);
    default: return cube_fail(c, CUBE_ERR_ARG, "own transforms need a power-of-two mesh of 64 to 2048");
  }
}
