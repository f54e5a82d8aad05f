// cube_ic.cu -- Zel'dovich initial conditions generated on the device, in the
// compressed state layout, following the steps of the reference's IC program
// (CUBEnu/work/utilities/initial_conditions.f90) with two stated substitutions:
//  * the CAMB transfer table is replaced by the Eisenstein & Hu (1998)
//    no-wiggle fitting formula, normalised to sigma_8 with the reference's
//    top-hat sum (:213-225) and grown with its Dgrow (:930-943);
//  * the gfortran random_number stream is replaced by a counter hash (the
//    murmur3 32-bit finaliser of seed and cell index), identical on every
//    device and launch shape.
// The rest is the reference's: Box-Muller on pairs along x (:292-300), the
// delta(k) scaling (:306-330), the discrete -4 pi/k^2 potential with its
// real-space correction (:433-503), Zel'dovich displacement and velocity by
// central differences of phi (:702-769), the per-cell mean velocity field and
// the atan velocity code of the residuals (:744-754), xp = floor(x/x_res)
// wrapped to izipx bytes (:741), pid = 1-based Lagrangian fine index
// (:757-761).  sigma_vi is the rms of the residual velocities / sqrt(3), the
// form update_xp uses every step (update_particle.f90:224).  Particles inside
// a cell are in Lagrangian order.
#include <cmath>
#include <vector>

#include "cube_internal.cuh"

namespace {

constexpr double kPi = 3.14159265358979323846;

// ---------------------------------------------------------------- host side
double eh_nowiggle(double k, double om, double h, double ob) {
  // Eisenstein & Hu (1998) zero-baryon-oscillation transfer, their eqs. 26, 28-31; k in h/Mpc
  const double theta = 2.7255 / 2.7;
  const double omh2 = om * h * h, obh2 = ob * h * h, fb = ob / om;
  const double s = 44.5 * std::log(9.83 / omh2) / std::sqrt(1.0 + 10.0 * std::pow(obh2, 0.75));
  const double alpha = 1.0 - 0.328 * std::log(431.0 * omh2) * fb + 0.38 * std::log(22.3 * omh2) * fb * fb;
  const double kmpc = k * h;
  const double gamma_eff = om * h * (alpha + (1.0 - alpha) / (1.0 + std::pow(0.43 * kmpc * s, 4)));
  const double q = k * theta * theta / gamma_eff;
  const double L0 = std::log(2.0 * std::exp(1.0) + 1.8 * q);
  const double C0 = 14.2 + 731.0 / (1.0 + 62.5 * q);
  return L0 / (L0 + C0 * q * q);
}

double dgrow(double a, double om, double ol) {
  // Carroll, Press & Turner growth, normalised to a = 1 (initial_conditions.f90:930-943)
  const double hsq = om / (a * a * a) + (1 - om - ol) / (a * a) + ol;
  const double oma = om / (a * a * a * hsq), ola = ol / hsq;
  const double g = 2.5 * om / (std::pow(om, 4.0 / 7) - ol + (1 + om / 2) * (1 + ol / 70));
  const double ga = 2.5 * oma / (std::pow(oma, 4.0 / 7) - ola + (1 + oma / 2) * (1 + ola / 70));
  return a * ga / g;
}

double vfactor(double a, double om, double ol) {
  // a^2 H for the Zel'dovich velocity (initial_conditions.f90:971-982, no neutrinos)
  const double lm = ol / om, km = (1 - om - ol) / om;
  const double H = 2.0 / (3.0 * std::sqrt(a * a * a)) * std::sqrt(1 + a * km + a * a * a * lm);
  return a * a * H;
}

// log k and log Delta^2(k) at a, normalised to sigma_8 over k <= kmax
void delta2_table(const cube_cosmology& cs, int nf, double a, std::vector<float>& lk, std::vector<float>& ld2) {
  const int nk = 1000;
  std::vector<double> k(nk), d2(nk), dk(nk);
  for (int i = 0; i < nk; i++) k[i] = std::pow(10.0, -4.0 + 6.0 * i / (nk - 1));
  for (int i = 0; i < nk; i++) {
    const double t = eh_nowiggle(k[i], cs.omega_m, cs.h0, cs.omega_b);
    d2[i] = t * t * std::pow(k[i], 3 + cs.n_s) / (2 * kPi * kPi);
  }
  dk[0] = k[1] / 2;
  for (int i = 1; i < nk - 1; i++) dk[i] = (k[i + 1] - k[i - 1]) / 2;
  dk[nk - 1] = k[nk - 1] - k[nk - 2];
  const double kmax = 2 * kPi * std::sqrt(3.0) * (nf / 2) / cs.box;
  double v8 = 0;
  for (int i = 0; i < nk; i++) {
    if (k[i] > kmax) continue;
    const double x = 8 * k[i], w = 3 * (std::sin(x) - std::cos(x) * x) / (x * x * x);
    v8 += d2[i] * w * w * dk[i] / k[i];
  }
  const double g = dgrow(a, cs.omega_m, cs.omega_l);
  const double norm = (double)cs.s8 * cs.s8 / v8 * g * g;
  lk.resize(nk);
  ld2.resize(nk);
  for (int i = 0; i < nk; i++) {
    lk[i] = (float)std::log(k[i]);
    ld2[i] = (float)std::log(d2[i] * norm);
  }
}

// ---------------------------------------------------------------- kernels
__host__ __device__ __forceinline__ uint32_t fmix32(uint32_t h) {
  h ^= h >> 16;
  h *= 0x85EBCA6Bu;
  h ^= h >> 13;
  h *= 0xC2B2AE35u;
  h ^= h >> 16;
  return h;
}
__device__ __forceinline__ float hash_uniform(uint64_t idx, uint32_t s) {
  uint32_t h = fmix32(fmix32((uint32_t)(idx ^ (uint64_t)s)) + s);
  return (float)(h >> 8) * (1.0f / 16777216.0f);
}

// Gaussian white noise: Box-Muller on the pairs (2i, 2i+1) along x (:292-300);
// rows of pitch floats
__global__ void k_ic_noise(float* r, int nf, int pitch, uint32_t s) {
  const int64_t npairs = (int64_t)nf * nf * (nf / 2);
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < npairs; q += (int64_t)gridDim.x * blockDim.x) {
    const int64_t row = q / (nf / 2);
    const int x = 2 * (int)(q - row * (nf / 2));
    const uint64_t i0 = (uint64_t)row * nf + x;
    const float u1 = hash_uniform(i0, s), u2 = hash_uniform(i0 + 1, s);
    const float rr = sqrtf(-2.0f * logf(1.0f - u2)), th = 2.0f * CUBE_PI_F * u1;
    float* o = r + row * pitch + x;
    o[0] = rr * cosf(th);
    o[1] = rr * sinf(th);
  }
}

// the discrete potential kernel -4 pi / khat^2 as a real half spectrum (:433-460)
__global__ void k_ic_kern(float2* ck, int nf) {
  const int nh = nf / 2 + 1;
  const int64_t n = (int64_t)nh * nf * nf;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int x = (int)(i % nh), y = (int)((i / nh) % nf), z = (int)(i / ((int64_t)nh * nf));
    const int kx = x, ky = y < (nf + 1) / 2 ? y : y - nf, kz = z < (nf + 1) / 2 ? z : z - nf;
    const float sx = 2.0f * sinf((float)kPi * kx / nf), sy = 2.0f * sinf((float)kPi * ky / nf),
                sz = 2.0f * sinf((float)kPi * kz / nf);
    const float ks = fmaxf(sx * sx + sy * sy + sz * sz, 1.0f / ((float)nf * nf));
    ck[i] = make_float2(i == 0 ? 0.f : -4.0f * (float)kPi / ks, 0.f);
  }
}

// real-space correction of the kernel (:462-503): beyond 8 cells shift by the
// mean at 8 cells plus 1/8, inside use -1/r, -2.5 at the origin
__global__ void k_ic_kern_correct(float* rk, int nf, float phi8) {
  const int64_t rows = (int64_t)nf * nf;
  const float inv = 1.0f / ((float)nf * nf * nf);  // the inverse transform's normalisation
  for (int64_t r = blockIdx.x; r < rows; r += gridDim.x) {
    const int y = (int)(r % nf), z = (int)(r / nf);
    const int cy = y < (nf + 1) / 2 ? y : y - nf, cz = z < (nf + 1) / 2 ? z : z - nf;
    for (int x = threadIdx.x; x < nf; x += blockDim.x) {
      const int cx = x < (nf + 1) / 2 ? x : x - nf;
      const float rr = sqrtf((float)(cx * cx + cy * cy + cz * cz));
      float* v = rk + r * (nf + 2) + x;
      const float val = *v * inv;
      *v = rr > 8.0f ? val - (phi8 + 0.125f) : (rr > 0.0f ? -1.0f / rr : -2.5f);
    }
  }
}

struct ScaleArgs {
  float2* ck;            // noise spectrum, scaled in place
  const float2* kk;      // corrected kernel spectrum (real part used)
  const float* lk;       // log k table
  const float* ld2;      // log Delta^2 table
  int ntab, nf;
  float kfac;            // 2 pi / box
  float* fout;           // when set: store the factor (times fscale) here instead of scaling ck
  float fscale;
};

// ck *= sqrt(Delta^2/(4 pi) * nf/kr) * nf/kr * KK  (:306-330, 505-541)
__global__ void k_ic_scale(ScaleArgs a) {
  const int nf = a.nf, nh = nf / 2 + 1;
  const int64_t n = (int64_t)nh * nf * nf;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    if (i == 0) {
      if (a.fout)
        a.fout[0] = 0.f;
      else
        a.ck[0] = make_float2(0.f, 0.f);
      continue;
    }
    const int x = (int)(i % nh), y = (int)((i / nh) % nf), z = (int)(i / ((int64_t)nh * nf));
    const int kx = x, ky = y < (nf + 1) / 2 ? y : y - nf, kz = z < (nf + 1) / 2 ? z : z - nf;
    const float kr = fmaxf(sqrtf((float)(kx * kx + ky * ky + kz * kz)), 1.0f);
    // log-log interpolation of the table (interp_tf, :895-916)
    float lx = logf(a.kfac * kr);
    lx = fminf(fmaxf(lx, a.lk[0]), a.lk[a.ntab - 1]);
    int lo = 0, hi = a.ntab - 1;
    while (hi - lo > 1) {
      const int mid = (lo + hi) >> 1;
      if (a.lk[mid] <= lx) lo = mid;
      else hi = mid;
    }
    const float t = (lx - a.lk[lo]) / (a.lk[hi] - a.lk[lo]);
    const float d2 = expf(a.ld2[lo] + (a.ld2[hi] - a.ld2[lo]) * t);
    const float f = sqrtf(d2 / (4.0f * (float)kPi) * ((float)nf / kr)) * ((float)nf / kr) * a.kk[i].x;
    if (a.fout) {
      a.fout[i] = f * a.fscale;
      continue;
    }
    const float2 c = a.ck[i];
    a.ck[i] = make_float2(c.x * f, c.y * f);
  }
}

struct PartArgs {
  const float* phi;  // padded, unnormalised inverse transform
  int nf, nc, nt, nnt, np_nc, step, ncell, izipx;
  float phiscale;    // 1/nf^3
  double vf;         // a^2 H
  int32_t* cid;      // cell id per Lagrangian particle
  void* xcode;       // 3 position codes per Lagrangian particle
  double* vel;       // 3 velocities per Lagrangian particle
  int32_t* counts;   // particles per cell
  unsigned int* vmax_bits;
};

// one thread per Lagrangian particle: displacement and velocity from central
// differences of phi at its fine lattice point (:702-769)
__global__ void k_ic_particles(PartArgs a, Geo g) {
  const int npd = a.nc * a.np_nc, nf = a.nf;
  const int64_t n = (int64_t)npd * npd * npd;
  float vm[3] = {0.f, 0.f, 0.f};
  for (int64_t l = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; l < n; l += (int64_t)gridDim.x * blockDim.x) {
    const int lx = (int)(l % npd), ly = (int)((l / npd) % npd), lz = (int)(l / ((int64_t)npd * npd));
    const int fx = a.step * lx, fy = a.step * ly, fz = a.step * lz;
    auto P = [&](int x, int y, int z) {
      return a.phi[mesh_idx(nf, wrap1(x, nf), wrap1(y, nf), wrap1(z, nf))] * a.phiscale;
    };
    const double gd[3] = {(double)(P(fx + 1, fy, fz) - P(fx - 1, fy, fz)), (double)(P(fx, fy + 1, fz) - P(fx, fy - 1, fz)),
                          (double)(P(fx, fy, fz + 1) - P(fx, fy, fz - 1))};
    const int li[3] = {lx, ly, lz};
    int cell[3];
    const int m = 1 << (8 * a.izipx);
    const double xres = 1.0 / m;
    for (int d = 0; d < 3; d++) {
      const double q = (double)li[d] / a.np_nc + 0.5 / a.ncell;
      double x = q - gd[d] / (8.0 * (double)CUBE_PI_F * a.ncell);
      x = x - a.nc * floor(x / a.nc);
      if (x >= a.nc) x -= a.nc;
      int c = (int)ceil(x) - 1;  // cell = ceiling(x), 1-based
      c = c < 0 ? c + a.nc : (c >= a.nc ? c - a.nc : c);
      cell[d] = c;
      long long xc = (long long)floor(x / xres);
      xc = ((xc % m) + m) % m;
      if (xc >= m / 2) xc -= m;
      if (a.izipx == 1)
        ((int8_t*)a.xcode)[3 * l + d] = (int8_t)xc;
      else
        ((int16_t*)a.xcode)[3 * l + d] = (int16_t)xc;
      const double v = -gd[d] / (8.0 * (double)CUBE_PI_F) * a.vf;
      a.vel[3 * l + d] = v;
      vm[d] = fmaxf(vm[d], (float)fabs(v));
    }
    const int32_t c = (int32_t)cell_id(g, cell[0], cell[1], cell[2]);
    a.cid[l] = c;
    atomicAdd(&a.counts[c], 1);
  }
  for (int d = 0; d < 3; d++) {
    float v = vm[d];
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    if ((threadIdx.x & 31) == 0) atomic_max_pos(&a.vmax_bits[d], v);
  }
}

// Thermal velocities of a massive-neutrino species (the sampling of
// CUBEnu/initial_conditions_mnu.f90:95-115): a speed q * fd with q drawn from
// the relativistic Fermi-Dirac distribution q^2/(e^q + 1) by inverse-CDF
// lookup with linear interpolation, an isotropic direction (cos theta uniform
// in [-1, 1), phi uniform in [0, 2 pi)), added to each particle's Zel'dovich
// velocity; vmax recomputed.  Three counter-hash streams per particle.
constexpr int kFdTab = 4096;
__global__ void k_ic_thermal(double* vel, int64_t n, const float* __restrict__ qtab, const float* __restrict__ ctab,
                             float fd, uint32_t s, unsigned int* vmax_bits) {
  float vm[3] = {0.f, 0.f, 0.f};
  for (int64_t l = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; l < n; l += (int64_t)gridDim.x * blockDim.x) {
    const float u = hash_uniform(3 * (uint64_t)l, s), uc = hash_uniform(3 * (uint64_t)l + 1, s),
                up = hash_uniform(3 * (uint64_t)l + 2, s);
    int lo = 0, hi = kFdTab - 1;  // ctab[lo] <= u < ctab[hi]
    while (hi - lo > 1) {
      const int mid = (lo + hi) >> 1;
      if (ctab[mid] <= u) lo = mid;
      else hi = mid;
    }
    const float t = (u - ctab[lo]) / fmaxf(ctab[hi] - ctab[lo], 1e-30f);
    const float q = qtab[lo] + (qtab[hi] - qtab[lo]) * t;
    const float sp = q * fd, ct = 2.0f * uc - 1.0f, st = sqrtf(fmaxf(1.0f - ct * ct, 0.f));
    float sn, cs;
    sincospif(2.0f * up, &sn, &cs);
    const double dv[3] = {(double)(sp * st * cs), (double)(sp * st * sn), (double)(sp * ct)};
    for (int d = 0; d < 3; d++) {
      const double v = vel[3 * l + d] + dv[d];
      vel[3 * l + d] = v;
      vm[d] = fmaxf(vm[d], (float)fabs(v));
    }
  }
  for (int d = 0; d < 3; d++) {
    float v = vm[d];
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    if ((threadIdx.x & 31) == 0) atomic_max_pos(&vmax_bits[d], v);
  }
}

// the Fermi-Dirac momentum CDF on kFdTab points of q in [0, 30]: the integral
// of q^2/(e^q+1) by composite Simpson on a 16x finer grid, normalised
void fd_table(std::vector<float>& q, std::vector<float>& c) {
  const int n = kFdTab, sub = 16;
  const double qmax = 30.0, h = qmax / ((double)(n - 1) * sub);
  auto f = [](double x) { return x * x / (std::exp(x) + 1.0); };
  std::vector<double> cum(n, 0.0);
  double acc = 0.0;
  for (int i = 1; i < n; i++) {
    const double a = (double)(i - 1) * sub * h;
    for (int k = 0; k < sub; k++) {
      const double x0 = a + k * h;
      acc += h / 6.0 * (f(x0) + 4.0 * f(x0 + h / 2) + f(x0 + h));
    }
    cum[i] = acc;
  }
  q.resize(n);
  c.resize(n);
  for (int i = 0; i < n; i++) {
    q[i] = (float)((double)i * qmax / (n - 1));
    c[i] = (float)(cum[i] / acc);
  }
  c[n - 1] = 1.0f;
}

// slot of each Lagrangian particle inside its cell (arbitrary order)
__global__ void k_ic_place(const int32_t* cid, int64_t n, const int64_t* cstart, int32_t* fill, int32_t* perm) {
  for (int64_t l = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; l < n; l += (int64_t)gridDim.x * blockDim.x) {
    const int32_t c = cid[l];
    perm[cstart[c] + atomicAdd(&fill[c], 1)] = (int32_t)l;
  }
}

// per cell: Lagrangian order (insertion sort of the cell's slots), then the
// mean velocity in that order (double sums, :744-748)
__global__ void k_ic_cells(const int64_t* cstart, int64_t ncells, int32_t* perm, const double* vel, float* vfield) {
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < ncells; c += (int64_t)gridDim.x * blockDim.x) {
    const int64_t p0 = cstart[c], p1 = cstart[c + 1];
    for (int64_t i = p0 + 1; i < p1; i++) {
      const int32_t v = perm[i];
      int64_t j = i - 1;
      while (j >= p0 && perm[j] > v) {
        perm[j + 1] = perm[j];
        j--;
      }
      perm[j + 1] = v;
    }
    double s[3] = {0.0, 0.0, 0.0};
    for (int64_t i = p0; i < p1; i++)
      for (int d = 0; d < 3; d++) s[d] += vel[3 * (int64_t)perm[i] + d];
    const double cnt = (double)(p1 > p0 ? p1 - p0 : 1);
    for (int d = 0; d < 3; d++) vfield[3 * c + d] = (float)(s[d] / cnt);
  }
}

struct GatherArgs {
  const int32_t* perm;
  const int32_t* cid;
  const void* xcode;
  const double* vel;
  const float* vfield;
  int izipx, npd, step, nf;
  void* xp;
  int32_t* pid;
  int32_t* pcell;
  double* res;      // residual velocities in the new order
  double* partial;  // per-block sums of res^2
};

// new order: position codes, pid, cell, residual velocities and their squares
__global__ void k_ic_gather(GatherArgs a, int64_t n) {
  double ss = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t l = a.perm[i];
    const int32_t c = a.cid[l];
    for (int d = 0; d < 3; d++) {
      if (a.izipx == 1)
        ((int8_t*)a.xp)[3 * i + d] = ((const int8_t*)a.xcode)[3 * l + d];
      else
        ((int16_t*)a.xp)[3 * i + d] = ((const int16_t*)a.xcode)[3 * l + d];
      const double r = a.vel[3 * l + d] - (double)a.vfield[3 * (int64_t)c + d];
      a.res[3 * i + d] = r;
      ss += r * r;
    }
    const int lx = (int)(l % a.npd), ly = (int)((l / a.npd) % a.npd), lz = (int)(l / ((int64_t)a.npd * a.npd));
    a.pid[i] = (int32_t)(a.step * lx + (int64_t)a.nf * (a.step * ly) + (int64_t)a.nf * a.nf * (a.step * lz) + 1);
    a.pcell[i] = c;
  }
  __shared__ double red[32];
  for (int o = 16; o > 0; o >>= 1) ss += __shfl_xor_sync(0xffffffffu, ss, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = ss;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += red[w];
    a.partial[blockIdx.x] = t;
  }
}

// velocity codes of the residuals (the reference's atan code, exact table encode)
__global__ void k_ic_encode(const double* res, int64_t n3, CodecView cv, int izipv, void* vp) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n3; i += (int64_t)gridDim.x * blockDim.x)
    store_code(vp, i, izipv, codec_encode(cv, res[i]));
}

// The corrected potential kernel's spectrum in kp (a padded nf^3 mesh, in
// place; :433-503) and the log Delta^2 table in dtab (2 x 1000 floats); fills
// sa for k_ic_scale except ck / fout.
int ic_kernel_spectrum(cube_ctx* c, int nf, cufftHandle r2c, cufftHandle c2r, float* kp, float* dtab,
                       const cube_cosmology& cs, double a, ScaleArgs& sa) {
  cudaStream_t s = c->stream;
  const int64_t nspec = (int64_t)(nf / 2 + 1) * nf * nf;
  k_ic_kern<<<cube_grid(nspec, 256), 256, 0, s>>>((float2*)kp, nf);
  CUBE_CUDA(c, cudaGetLastError());
  CUBE_FFT(c, cufftExecC2R(c2r, (cufftComplex*)kp, kp));
  {  // phi8: the mean of the six points at 8 cells on the axes
    auto at_ = [nf](int64_t x, int64_t y, int64_t z) { return x + (int64_t)(nf + 2) * (y + (int64_t)nf * z); };
    const int64_t at[6] = {at_(8, 0, 0), at_(0, 8, 0), at_(0, 0, 8), at_(nf - 8, 0, 0), at_(0, nf - 8, 0), at_(0, 0, nf - 8)};
    float h[6];
    for (int i = 0; i < 6; i++)
      CUBE_CUDA(c, cudaMemcpyAsync(&h[i], kp + at[i], 4, cudaMemcpyDeviceToHost, s));
    CUBE_CUDA(c, cudaStreamSynchronize(s));
    const float inv = 1.0f / ((float)nf * nf * nf);
    float phi8 = 0.f;
    for (int i = 0; i < 6; i++) phi8 += h[i] * inv;
    phi8 /= 6.0f;
    k_ic_kern_correct<<<cube_grid((int64_t)nf * nf, 1, 8), 256, 0, s>>>(kp, nf, phi8);
    CUBE_CUDA(c, cudaGetLastError());
  }
  CUBE_FFT(c, cufftExecR2C(r2c, kp, (cufftComplex*)kp));
  std::vector<float> lk, ld2;
  delta2_table(cs, nf, a, lk, ld2);
  CUBE_CUDA(c, cudaMemcpyAsync(dtab, lk.data(), 4 * lk.size(), cudaMemcpyHostToDevice, s));
  CUBE_CUDA(c, cudaMemcpyAsync(dtab + lk.size(), ld2.data(), 4 * ld2.size(), cudaMemcpyHostToDevice, s));
  CUBE_CUDA(c, cudaStreamSynchronize(s));  // the host tables go out of scope
  sa = ScaleArgs{nullptr, (const float2*)kp, dtab, dtab + lk.size(), (int)lk.size(), nf, (float)(2 * kPi / cs.box),
                 nullptr, 1.0f};
  return CUBE_OK;
}

}  // namespace

int cube_ic_filter(cube_ctx* c, const cube_cosmology& cs, double a, int n, cufftHandle r2c, cufftHandle c2r,
                   float* scratch, float* dtab, float* filter) {
  ScaleArgs sa;
  int r = ic_kernel_spectrum(c, n, r2c, c2r, scratch, dtab, cs, a, sa);
  if (r) return r;
  sa.fout = filter;
  sa.fscale = 1.0f / ((float)n * (float)n * (float)n);
  k_ic_scale<<<cube_grid((int64_t)(n / 2 + 1) * n * n, 256), 256, 0, c->stream>>>(sa);
  CUBE_CUDA(c, cudaGetLastError());
  return CUBE_OK;
}

uint32_t cube_ic_seed(uint32_t seed) { return fmix32((uint32_t)((uint64_t)seed * 0x9E3779B1ull + 0x7F4A7C15ull)); }

void cube_ic_noise(float* r, int n, int pitch, uint32_t seed, cudaStream_t s) {
  k_ic_noise<<<cube_grid((int64_t)n * n * (n / 2), 256), 256, 0, s>>>(r, n, pitch, cube_ic_seed(seed));
}

double cube_ic_vfactor(double a, double om, double ol) { return vfactor(a, om, ol); }

static int ic_impl(cube_ctx* c, const cube_cosmology* cs, float z_init, uint32_t seed, float m_nu_ev,
                   uint32_t thermal_seed, float* sigma_vi, float* vmax);

extern "C" int cube_ic_zeldovich(cube_ctx* c, const cube_cosmology* cs, float z_init, uint32_t seed, float* sigma_vi,
                                 float* vmax) {
  return ic_impl(c, cs, z_init, seed, 0.f, 0u, sigma_vi, vmax);
}

extern "C" int cube_ic_zeldovich_nu(cube_ctx* c, const cube_cosmology* cs, float z_init, uint32_t seed, float m_nu_ev,
                                    uint32_t thermal_seed, float* sigma_vi, float* vmax) {
  if (!(m_nu_ev > 0.f)) return cube_fail(c, CUBE_ERR_ARG, "the neutrino mass must be positive");
  return ic_impl(c, cs, z_init, seed, m_nu_ev, thermal_seed, sigma_vi, vmax);
}

static int ic_impl(cube_ctx* c, const cube_cosmology* cs, float z_init, uint32_t seed, float m_nu_ev,
                   uint32_t thermal_seed, float* sigma_vi, float* vmax) {
  if (!c || !cs) return CUBE_ERR_ARG;
  const cube_params& p = c->p;
  if (cs->np_nc < 1 || p.ncell % cs->np_nc) return cube_fail(c, CUBE_ERR_ARG, "np_nc must divide ncell");
  const int nf = c->nf, nc = p.nc, npd = nc * cs->np_nc;
  const int64_t n = (int64_t)npd * npd * npd;
  if (n > p.np_max) return cube_fail(c, CUBE_ERR_IMAGE_OVERFLOW, "np_max is below the particle count of the grid");
  if (nf % 2) return cube_fail(c, CUBE_ERR_ARG, "fine mesh must be even");
  // FP64 velocities and residuals (24 bytes per particle each) live in two
  // force planes when they fit (a particle per 8 fine cells and sparser),
  // else in buffers of their own for the duration of the call
  const bool fits = (size_t)24 * n <= sizeof(float) * (size_t)(nf + 2) * nf * nf;
  struct Scratch {
    void* p = nullptr;
    ~Scratch() {
      if (p) cudaFree(p);
    }
  } own;
  if (!fits) {
    cudaError_t e = cudaMalloc(&own.p, (size_t)48 * n);
    if (e != cudaSuccess) return cube_fail(c, CUBE_ERR_NOMEM, "initial-condition velocity scratch");
  }
  CUBE_CUDA(c, cudaSetDevice(c->device));
  if (int r = cube_copy_join(c)) return r;
  if (int r = cube_upload_join(c)) return r;
  cudaStream_t s = c->stream;
  const double a = 1.0 / (1.0 + z_init);
  const int64_t nspec = (int64_t)(nf / 2 + 1) * nf * nf;
  const int k = c->cur, alt = 1 - k;
  // 1. noise and its spectrum
  cube_ic_noise(c->rho_f, nf, nf + 2, seed, s);
  CUBE_CUDA(c, cudaGetLastError());
  CUBE_FFT(c, cufftExecR2C(c->plan_f_r2c, c->rho_f, (cufftComplex*)c->rho_f));
  // 2. corrected potential kernel in force plane 0, tables in force plane 1
  float* kp = c->force_f[0];
  float* dtab = reinterpret_cast<float*>(c->force_f[1]);
  ScaleArgs sa;
  int r = ic_kernel_spectrum(c, nf, c->plan_f_r2c, c->plan_f_c2r, kp, dtab, *cs, a, sa);
  if (r) return r;
  // 3. scaled spectrum times the kernel, then phi
  sa.ck = (float2*)c->rho_f;
  k_ic_scale<<<cube_grid(nspec, 256), 256, 0, s>>>(sa);
  CUBE_CUDA(c, cudaGetLastError());
  CUBE_FFT(c, cufftExecC2R(c->plan_f_c2r, (cufftComplex*)c->rho_f, c->rho_f));
  // 4. particles on the Lagrangian grid
  int32_t* cid = c->dest;
  double* vel = fits ? reinterpret_cast<double*>(c->force_f[1]) : static_cast<double*>(own.p);
  CUBE_CUDA(c, cudaMemsetAsync(c->rhoc[k], 0, 4 * (size_t)c->ncells, s));
  CUBE_CUDA(c, cudaMemsetAsync(c->dstats, 0, sizeof(DevStats), s));
  PartArgs pa{c->rho_f, nf, nc, c->nt, p.nnt, cs->np_nc, p.ncell / cs->np_nc, p.ncell, p.izipx,
              1.0f / ((float)nf * nf * nf), vfactor(a, cs->omega_m, cs->omega_l), cid, c->xp[alt], vel, c->rhoc[k],
              c->dstats->vmax_bits};
  k_ic_particles<<<cube_grid(n, 256), 256, 0, s>>>(pa, make_geo(c));
  CUBE_CUDA(c, cudaGetLastError());
  if (m_nu_ev > 0.f) {
    // thermal speeds: k_B T_nu c / m_nu = 50.2476 km/s / m_nu[eV] / a
    // (initial_conditions_mnu.f90:33), in simulation units through
    // vsim2phys = (150/a) box sqrt(omega_m) / nf_global (initial_conditions.f90:175)
    const double vsim2phys = 150.0 / a * (double)cs->box * std::sqrt((double)cs->omega_m) / (double)nf;
    const float fd = (float)(50.2476 / (double)m_nu_ev / a / vsim2phys);
    std::vector<float> qt, ct;
    fd_table(qt, ct);
    float* tab = reinterpret_cast<float*>(c->force_f[0]);  // the kernel spectrum is no longer needed
    CUBE_CUDA(c, cudaMemcpyAsync(tab, qt.data(), 4 * qt.size(), cudaMemcpyHostToDevice, s));
    CUBE_CUDA(c, cudaMemcpyAsync(tab + kFdTab, ct.data(), 4 * ct.size(), cudaMemcpyHostToDevice, s));
    CUBE_CUDA(c, cudaMemsetAsync(c->dstats->vmax_bits, 0, 12, s));
    k_ic_thermal<<<cube_grid(n, 256), 256, 0, s>>>(vel, n, tab, tab + kFdTab, fd, cube_ic_seed(thermal_seed ^ 0x5bd1e995u),
                                                   c->dstats->vmax_bits);
    CUBE_CUDA(c, cudaGetLastError());
    CUBE_CUDA(c, cudaStreamSynchronize(s));  // the host tables go out of scope
  }
  r = cube_scan_counts(c, c->rhoc[k], c->cstart[k], c->ncells);
  if (r) return r;
  int32_t* fill = reinterpret_cast<int32_t*>(c->rank);
  CUBE_CUDA(c, cudaMemsetAsync(fill, 0, 4 * (size_t)c->ncells, s));
  k_ic_place<<<cube_grid(n, 256), 256, 0, s>>>(cid, n, c->cstart[k], fill, c->perm);
  k_ic_cells<<<cube_grid(c->ncells, 128), 128, 0, s>>>(c->cstart[k], c->ncells, c->perm, vel, c->vfield[k]);
  CUBE_CUDA(c, cudaGetLastError());
  // 5. the new order, residuals and sigma
  double* res = fits ? reinterpret_cast<double*>(c->force_f[2]) : static_cast<double*>(own.p) + 3 * n;
  const int nb = cube_grid(n, 256, 4);
  double* part = reinterpret_cast<double*>(c->rho_f);  // phi is no longer needed
  GatherArgs ga{c->perm, cid, c->xp[alt], vel, c->vfield[k], p.izipx, npd, p.ncell / cs->np_nc, nf,
                c->xp[k], c->pid[k], c->pcell[k], res, part};
  k_ic_gather<<<nb, 256, 0, s>>>(ga, n);
  CUBE_CUDA(c, cudaGetLastError());
  std::vector<double> hp(nb);
  CUBE_CUDA(c, cudaMemcpyAsync(hp.data(), part, 8 * (size_t)nb, cudaMemcpyDeviceToHost, s));
  r = cube_stats_fetch(c);
  if (r) return r;
  double ss = 0.0;
  for (int b = 0; b < nb; b++) ss += hp[b];
  const float sig = (float)(std::sqrt(ss / (double)n) / std::sqrt(3.0));
  if (!(sig > 0.f)) return cube_fail(c, CUBE_ERR_NONFINITE, "residual velocities vanish");
  float vm[3];
  for (int d = 0; d < 3; d++) vm[d] = bits_float(c->hstats->vmax_bits[d]);
  // 6. velocity codes with the codec of sigma
  CodecView cv;
  r = cube_codec_pair(c, sig, sig, &cv, nullptr);
  if (r) return r;
  k_ic_encode<<<cube_grid(3 * n, 256), 256, 0, s>>>(res, 3 * n, cv, p.izipv, c->vp[k]);
  CUBE_CUDA(c, cudaGetLastError());
  CUBE_CUDA(c, cudaStreamSynchronize(s));
  c->np = n;
  c->npglobal = n;
  c->have_state = true;
  c->sigma_vi = c->sigma_vi_new = sig;
  for (int d = 0; d < 3; d++) c->vmax_prev[d] = 0.f;
  if (sigma_vi) *sigma_vi = sig;
  if (vmax)
    for (int d = 0; d < 3; d++) vmax[d] = vm[d];
  return CUBE_OK;
}
