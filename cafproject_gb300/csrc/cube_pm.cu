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
// K*0.25*pi*ksin_d/sum(ksin^2)/Im(FFT(raw)).
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
struct DepArgs {
  Geo g;
  int64_t np;
  const void* xp;
  const int32_t* pcell;
  float mass;
  float* rho;
  double* mass_sum;
};

__global__ void k_deposit_fine(DepArgs a) {
  const Geo& g = a.g;
  double msum = 0;
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < a.np; p += (int64_t)gridDim.x * blockDim.x) {
    int gc[3];
    cell_coords(g, a.pcell[p], gc[0], gc[1], gc[2]);
    int i1[3], i2[3];
    float d1[3], d2[3];
    for (int d = 0; d < 3; d++) {
      int T = gc[d] / g.nt, L = gc[d] - T * g.nt + 1;
      float tx = fine_tempx(g.ncell, L, load_code(a.xp, 3 * p + d, g.izipx), g.izipx);
      float fl = floorf(tx);
      d1[d] = __fsub_rn(__fadd_rn(fl, 1.0f), tx);
      d2[d] = __fsub_rn(1.0f, d1[d]);
      int base = T * g.nt * g.ncell + (int)fl;  // global fine cell of idx1
      i1[d] = wrapi(base, g.nf);
      i2[d] = wrapi(base + 1, g.nf);
    }
    float m = a.mass;
    float w[8];
    w[0] = __fmul_rn(__fmul_rn(__fmul_rn(d1[0], d1[1]), d1[2]), m);
    w[1] = __fmul_rn(__fmul_rn(__fmul_rn(d2[0], d1[1]), d1[2]), m);
    w[2] = __fmul_rn(__fmul_rn(__fmul_rn(d1[0], d2[1]), d1[2]), m);
    w[3] = __fmul_rn(__fmul_rn(__fmul_rn(d1[0], d1[1]), d2[2]), m);
    w[4] = __fmul_rn(__fmul_rn(__fmul_rn(d1[0], d2[1]), d2[2]), m);
    w[5] = __fmul_rn(__fmul_rn(__fmul_rn(d2[0], d1[1]), d2[2]), m);
    w[6] = __fmul_rn(__fmul_rn(__fmul_rn(d2[0], d2[1]), d1[2]), m);
    w[7] = __fmul_rn(__fmul_rn(__fmul_rn(d2[0], d2[1]), d2[2]), m);
    int n = g.nf;
    atomicAdd(&a.rho[mesh_idx(n, i1[0], i1[1], i1[2])], w[0]);
    atomicAdd(&a.rho[mesh_idx(n, i2[0], i1[1], i1[2])], w[1]);
    atomicAdd(&a.rho[mesh_idx(n, i1[0], i2[1], i1[2])], w[2]);
    atomicAdd(&a.rho[mesh_idx(n, i1[0], i1[1], i2[2])], w[3]);
    atomicAdd(&a.rho[mesh_idx(n, i1[0], i2[1], i2[2])], w[4]);
    atomicAdd(&a.rho[mesh_idx(n, i2[0], i1[1], i2[2])], w[5]);
    atomicAdd(&a.rho[mesh_idx(n, i2[0], i2[1], i1[2])], w[6]);
    atomicAdd(&a.rho[mesh_idx(n, i2[0], i2[1], i2[2])], w[7]);
    for (int k = 0; k < 8; k++) msum += (double)w[k];
  }
  for (int o = 16; o > 0; o >>= 1) msum += __shfl_xor_sync(0xffffffffu, msum, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(a.mass_sum, msum);
}

// coarse CIC with the -0.5 shift in the tile frame (pm.f90:221)
__global__ void k_deposit_coarse(DepArgs a) {
  const Geo& g = a.g;
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < a.np; p += (int64_t)gridDim.x * blockDim.x) {
    int gc[3];
    cell_coords(g, a.pcell[p], gc[0], gc[1], gc[2]);
    int i1[3], i2[3];
    float d1[3], d2[3];
    for (int d = 0; d < 3; d++) {
      int T = gc[d] / g.nt, L = gc[d] - T * g.nt + 1;
      float tx = coarse_tempx(L, load_code(a.xp, 3 * p + d, g.izipx), g.izipx);
      float fl = floorf(tx);
      d1[d] = __fsub_rn(__fadd_rn(fl, 1.0f), tx);
      d2[d] = __fsub_rn(1.0f, d1[d]);
      int base = T * g.nt + (int)fl;
      i1[d] = wrapi(base, g.nc);
      i2[d] = wrapi(base + 1, g.nc);
    }
    float m = a.mass;
    int n = g.nc;
    atomicAdd(&a.rho[mesh_idx(n, i1[0], i1[1], i1[2])], __fmul_rn(__fmul_rn(__fmul_rn(d1[0], d1[1]), d1[2]), m));
    atomicAdd(&a.rho[mesh_idx(n, i2[0], i1[1], i1[2])], __fmul_rn(__fmul_rn(__fmul_rn(d2[0], d1[1]), d1[2]), m));
    atomicAdd(&a.rho[mesh_idx(n, i1[0], i2[1], i1[2])], __fmul_rn(__fmul_rn(__fmul_rn(d1[0], d2[1]), d1[2]), m));
    atomicAdd(&a.rho[mesh_idx(n, i1[0], i1[1], i2[2])], __fmul_rn(__fmul_rn(__fmul_rn(d1[0], d1[1]), d2[2]), m));
    atomicAdd(&a.rho[mesh_idx(n, i1[0], i2[1], i2[2])], __fmul_rn(__fmul_rn(__fmul_rn(d1[0], d2[1]), d2[2]), m));
    atomicAdd(&a.rho[mesh_idx(n, i2[0], i1[1], i2[2])], __fmul_rn(__fmul_rn(__fmul_rn(d2[0], d1[1]), d2[2]), m));
    atomicAdd(&a.rho[mesh_idx(n, i2[0], i2[1], i1[2])], __fmul_rn(__fmul_rn(__fmul_rn(d2[0], d2[1]), d1[2]), m));
    atomicAdd(&a.rho[mesh_idx(n, i2[0], i2[1], i2[2])], __fmul_rn(__fmul_rn(__fmul_rn(d2[0], d2[1]), d2[2]), m));
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

// maxval(sum(force**2,1)) over the mesh (pm.f90:126, 315)
__global__ void k_f2max(const float* __restrict__ f0, const float* __restrict__ f1, const float* __restrict__ f2,
                        int n, unsigned int* __restrict__ out) {
  int64_t rows = (int64_t)n * n;
  float m = 0.f;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < rows * n; i += (int64_t)gridDim.x * blockDim.x) {
    int64_t r = i / n;
    int x = (int)(i - r * n);
    int64_t j = r * (n + 2) + x;
    float a = f0[j], b = f1[j], c = f2[j];
    float s = __fadd_rn(__fadd_rn(__fmul_rn(a, a), __fmul_rn(b, b)), __fmul_rn(c, c));
    m = fmaxf(m, s);
  }
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomic_max_pos(out, m);
}

// ------------------------------------------------------------------- kicks
struct KickArgs {
  Geo g;
  int64_t np;
  const void* xp;
  void* vp;
  const int32_t* pcell;
  const float* vfield;
  const float* f[3];
  const double* dec;
  int nvbin;
  double vc_out;
  float a_mid, dt;
  unsigned int* vmax_bits;  // coarse kick only
};

template <bool kFine>
__global__ void k_kick(KickArgs a) {
  const Geo& g = a.g;
  float vm[3] = {0.f, 0.f, 0.f};
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < a.np; p += (int64_t)gridDim.x * blockDim.x) {
    int64_t cell = a.pcell[p];
    int gc[3];
    cell_coords(g, cell, gc[0], gc[1], gc[2]);
    int i1[3], i2[3];
    float d1[3], d2[3];
    int n = kFine ? g.nf : g.nc;
    for (int d = 0; d < 3; d++) {
      int T = gc[d] / g.nt, L = gc[d] - T * g.nt + 1;
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
      d1[d] = __fsub_rn(__fadd_rn(fl, 1.0f), tx);
      d2[d] = __fsub_rn(1.0f, d1[d]);
      i1[d] = wrapi(base, n);
      i2[d] = wrapi(base + 1, n);
    }
    int64_t c111 = mesh_idx(n, i1[0], i1[1], i1[2]), c211 = mesh_idx(n, i2[0], i1[1], i1[2]);
    int64_t c121 = mesh_idx(n, i1[0], i2[1], i1[2]), c112 = mesh_idx(n, i1[0], i1[1], i2[2]);
    int64_t c122 = mesh_idx(n, i1[0], i2[1], i2[2]), c212 = mesh_idx(n, i2[0], i1[1], i2[2]);
    int64_t c221 = mesh_idx(n, i2[0], i2[1], i1[2]), c222 = mesh_idx(n, i2[0], i2[1], i2[2]);
    for (int d = 0; d < 3; d++) {
      const float* F = a.f[d];
      int code = load_code(a.vp, 3 * p + d, g.izipv);
      double v = a.dec[code + a.nvbin / 2];
      v = __dadd_rn(v, (double)kick_term(F[c111], a.a_mid, a.dt, d1[0], d1[1], d1[2]));
      v = __dadd_rn(v, (double)kick_term(F[c211], a.a_mid, a.dt, d2[0], d1[1], d1[2]));
      v = __dadd_rn(v, (double)kick_term(F[c121], a.a_mid, a.dt, d1[0], d2[1], d1[2]));
      v = __dadd_rn(v, (double)kick_term(F[c112], a.a_mid, a.dt, d1[0], d1[1], d2[2]));
      v = __dadd_rn(v, (double)kick_term(F[c122], a.a_mid, a.dt, d1[0], d2[1], d2[2]));
      v = __dadd_rn(v, (double)kick_term(F[c212], a.a_mid, a.dt, d2[0], d1[1], d2[2]));
      v = __dadd_rn(v, (double)kick_term(F[c221], a.a_mid, a.dt, d2[0], d2[1], d1[2]));
      v = __dadd_rn(v, (double)kick_term(F[c222], a.a_mid, a.dt, d2[0], d2[1], d2[2]));
      if (!kFine) {
        // vmax=max(vmax,abs(vreal+vfield)) (pm.f90:349), real(4) result
        double w = fabs(__dadd_rn(v, (double)a.vfield[3 * cell + d]));
        vm[d] = fmaxf(vm[d], __double2float_rn(w));
      }
      store_code(a.vp, 3 * p + d, g.izipv, v_encode(v, a.vc_out, a.nvbin));
    }
  }
  if (!kFine) {
    for (int d = 0; d < 3; d++) {
      float m = vm[d];
      for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
      if ((threadIdx.x & 31) == 0) atomic_max_pos(&a.vmax_bits[d], m);
    }
  }
}

double vcoef_h(float sigma) {
  float s = std::sqrt(CUBE_PI_F / 2.0f);
  return (double)s / ((double)sigma * 2.5);
}

}  // namespace

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
int cube_fine_density_impl(cube_ctx* c, cube_stats* st) {
  cudaStream_t s = c->stream;
  Geo g = make_geo(c);
  int64_t nfh = c->nf / 2 + 1;
  int64_t nspec = nfh * c->nf * (int64_t)c->nf;
  CUBE_CUDA(c, cudaMemsetAsync(c->rho_f, 0, 8 * nspec, s));
  CUBE_CUDA(c, cudaMemsetAsync(c->dstats, 0, sizeof(DevStats), s));
  DepArgs a{g, c->np, c->xp[c->cur], c->pcell[c->cur], c->p.mass_p, c->rho_f, &c->dstats->testrhof};
  cube_phase_begin(c, PH_F_DEPOSIT);
  k_deposit_fine<<<cube_grid(c->np, 256), 256, 0, s>>>(a);
  cube_phase_end(c, PH_F_DEPOSIT);
  CUBE_CUDA(c, cudaGetLastError());
  if (st) {
    int r = cube_stats_fetch(c);
    if (r) return r;
    st->testrhof = c->hstats->testrhof;
  }
  return CUBE_OK;
}

int cube_fine_forces_impl(cube_ctx* c, cube_stats* st) {
  cudaStream_t s = c->stream;
  int64_t nfh = c->nf / 2 + 1;
  int64_t nspec = nfh * c->nf * (int64_t)c->nf;
  int r0 = cube_fine_density_impl(c, nullptr);
  if (r0) return r0;
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
  k_f2max<<<cube_grid(c->nfine, 256), 256, 0, s>>>(c->force_f[0], c->force_f[1], c->force_f[2], c->nf,
                                                   &c->dstats->f2_fine_bits);
  cube_phase_end(c, PH_F_F2MAX);
  CUBE_CUDA(c, cudaGetLastError());
  if (st) {
    int r = cube_stats_fetch(c);
    if (r) return r;
    st->f2_max_fine = bits_float(c->hstats->f2_fine_bits);
    st->testrhof = c->hstats->testrhof;
  }
  return CUBE_OK;
}

int cube_fine_kick_impl(cube_ctx* c, float a_mid, float dt) {
  int r = cube_ensure_decode(c, c->dec_old, c->sigma_vi, c->dec_old_sigma);
  if (r) return r;
  KickArgs k{};
  k.g = make_geo(c);
  k.np = c->np;
  k.xp = c->xp[c->cur];
  k.vp = c->vp[c->cur];
  k.pcell = c->pcell[c->cur];
  k.vfield = c->vfield[c->cur];
  for (int d = 0; d < 3; d++) k.f[d] = c->force_f[d];
  k.dec = c->dec_old;
  k.nvbin = c->nvbin;
  k.vc_out = vcoef_h(c->sigma_vi_new);
  k.a_mid = a_mid;
  k.dt = dt;
  k.vmax_bits = nullptr;
  cube_phase_begin(c, PH_F_KICK);
  k_kick<true><<<cube_grid(c->np, 256), 256, 0, c->stream>>>(k);
  cube_phase_end(c, PH_F_KICK);
  CUBE_CUDA(c, cudaGetLastError());
  return CUBE_OK;
}

// --------------------------------------------------------------- coarse
int cube_coarse_density_impl(cube_ctx* c, cube_stats* st) {
  cudaStream_t s = c->stream;
  Geo g = make_geo(c);
  int nc = c->p.nc;
  int64_t nch = nc / 2 + 1;
  int64_t cspec = nch * nc * (int64_t)nc;
  CUBE_CUDA(c, cudaMemsetAsync(c->rho_c, 0, 8 * cspec, s));
  CUBE_CUDA(c, cudaMemsetAsync(&c->dstats->f2_coarse_bits, 0, 4, s));
  DepArgs a{g, c->np, c->xp[c->cur], c->pcell[c->cur], c->p.mass_p, c->rho_c, nullptr};
  cube_phase_begin(c, PH_C_DEPOSIT);
  k_deposit_coarse<<<cube_grid(c->np, 256), 256, 0, s>>>(a);
  cube_phase_end(c, PH_C_DEPOSIT);
  CUBE_CUDA(c, cudaGetLastError());
  (void)st;
  return CUBE_OK;
}

int cube_coarse_forces_impl(cube_ctx* c, cube_stats* st) {
  cudaStream_t s = c->stream;
  int nc = c->p.nc;
  int64_t nch = nc / 2 + 1;
  int64_t cspec = nch * nc * (int64_t)nc;
  int r0 = cube_coarse_density_impl(c, nullptr);
  if (r0) return r0;
  cube_phase_begin(c, PH_C_FFT);
  CUBE_FFT(c, cufftExecR2C(c->plan_c_r2c, c->rho_c, (cufftComplex*)c->rho_c));
  k_green3<<<cube_grid(cspec, 256), 256, 0, s>>>((const float2*)c->rho_c, c->kern_c, cspec, (float2*)c->force_c[0],
                                                  (float2*)c->force_c[1], (float2*)c->force_c[2]);
  for (int d = 0; d < 3; d++)
    CUBE_FFT(c, cufftExecC2R(c->plan_c_c2r, (cufftComplex*)c->force_c[d], c->force_c[d]));
  k_f2max<<<cube_grid((int64_t)nc * nc * nc, 256), 256, 0, s>>>(c->force_c[0], c->force_c[1], c->force_c[2], nc,
                                                                 &c->dstats->f2_coarse_bits);
  cube_phase_end(c, PH_C_FFT);
  CUBE_CUDA(c, cudaGetLastError());
  if (st) {
    int r = cube_stats_fetch(c);
    if (r) return r;
    st->f2_max_coarse = bits_float(c->hstats->f2_coarse_bits);
  }
  return CUBE_OK;
}

int cube_coarse_kick_impl(cube_ctx* c, float a_mid, float dt, cube_stats* st) {
  int r = cube_ensure_decode(c, c->dec_old, c->sigma_vi, c->dec_old_sigma);
  if (r) return r;
  CUBE_CUDA(c, cudaMemsetAsync(c->dstats->vmax_bits, 0, 12, c->stream));
  KickArgs k{};
  k.g = make_geo(c);
  k.np = c->np;
  k.xp = c->xp[c->cur];
  k.vp = c->vp[c->cur];
  k.pcell = c->pcell[c->cur];
  k.vfield = c->vfield[c->cur];
  for (int d = 0; d < 3; d++) k.f[d] = c->force_c[d];
  k.dec = c->dec_old;
  k.nvbin = c->nvbin;
  k.vc_out = vcoef_h(c->sigma_vi);
  k.a_mid = a_mid;
  k.dt = dt;
  k.vmax_bits = c->dstats->vmax_bits;
  cube_phase_begin(c, PH_C_KICK);
  k_kick<false><<<cube_grid(c->np, 256), 256, 0, c->stream>>>(k);
  cube_phase_end(c, PH_C_KICK);
  CUBE_CUDA(c, cudaGetLastError());
  if (st) {
    r = cube_stats_fetch(c);
    if (r) return r;
    for (int d = 0; d < 3; d++) st->vmax[d] = bits_float(c->hstats->vmax_bits[d]);
    st->f2_max_coarse = bits_float(c->hstats->f2_coarse_bits);
  }
  return CUBE_OK;
}
