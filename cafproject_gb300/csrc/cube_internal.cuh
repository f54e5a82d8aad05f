// cube_internal.cuh -- context, layouts and exact-arithmetic device helpers
// shared by the GB300 kernels of the CUBE per-step path.
//
// Device layout (one image, nn=1, all resident in HBM):
//   particles  xp[3*np] / vp[3*np] (reference AoS bytes), pid[np]; sorted by
//              cell id c = ix + nt*(iy + nt*(iz + nt*tile)),
//              tile = tx + nnt*(ty + nnt*tz)  (the reference disjoint order)
//   cells      rhoc[c] int32, vfield[3*c] float, cstart[c] int64 (exclusive scan)
//   fine mesh  nf^3 periodic (nf = nc*ncell) in cuFFT's padded in-place layout
//              (row stride nf+2 floats); one global grid replaces the
//              reference's per-tile nfe^3 boxes: the fine kernel reaches 15
//              cells < nfb=24, so the tile force equals the periodic one.
//   coarse     nc^3 periodic, same padded layout.
//
// Exactness: the FP32/FP64 sequences that set integer state (decode, kick
// accumulation, drift, encode) use explicit round-to-nearest intrinsics so
// no FMA contraction changes their bits.
#pragma once
#include <cuda_runtime.h>
#include <cufft.h>
#include <stdint.h>

#include <string>

#include "../../include/cube_gpu.h"

#define CUBE_PI_F 3.14159274101257324f  // pi=4*atan(1.) in real(4), parameters.f90:67

struct DevStats {
  // update_x
  unsigned long long nlost, ndup, nfar, max_tile;
  int max_disp;
  int flags;
  // particle_mesh / pp
  unsigned int f2_fine_bits, f2_coarse_bits, f2_pp_bits;
  unsigned int vmax_bits[3];
  unsigned long long npairs, itest1;
  unsigned long long ndup_list;  // entries in the extra-copy list
  double testrhof, testrhoc;
};

struct cube_ctx {
  cube_params p{};
  int device = 0;
  cudaStream_t stream = nullptr;
  std::string err;
  // derived sizes
  int nt = 0, nf = 0, ntiles = 0, nvbin = 0;
  int64_t ncells = 0;  // nc^3
  int64_t nfine = 0;   // nf^3
  // state (ping-pong between update_x calls)
  int cur = 0;
  int64_t np = 0;
  bool have_state = false;
  void* xp[2] = {nullptr, nullptr};
  void* vp[2] = {nullptr, nullptr};
  int32_t* pid[2] = {nullptr, nullptr};
  int32_t* pcell[2] = {nullptr, nullptr};  // cell id of each particle (derived index)
  int64_t npglobal = 0;                    // sim%npglobal (count at upload)
  int32_t* rhoc[2] = {nullptr, nullptr};
  float* vfield[2] = {nullptr, nullptr};
  int64_t* cstart[2] = {nullptr, nullptr};
  // update_x scratch
  int32_t* dest = nullptr;      // primary destination cell per particle (-1: none)
  uint8_t* dframe = nullptr;    // frame of the primary copy: (ox+1)+3(oy+1)+9(oz+1), o in tiles
  uint32_t* rank = nullptr;     // rank of the primary copy in its destination
  int4* xtra = nullptr;         // extra copies: (particle, dest cell, rank, -)
  int64_t xtra_cap = 0;
  void* scan_tmp = nullptr;
  size_t scan_tmp_bytes = 0;
  double* red_tmp = nullptr;    // block partial sums for sigma statistics
  int red_blocks = 0;
  // velocity code tables
  float* tan_tab = nullptr;     // float(tan(pi*v/(nvbin-1))) for v in [-nvbin/2, nvbin/2)
  double* dec_old = nullptr;    // decode table for sigma_vi
  double* dec_new = nullptr;    // decode table for sigma_vi_new
  float dec_old_sigma = -1.f, dec_new_sigma = -1.f;
  float sigma_vi = 0.f, sigma_vi_new = 0.f;
  // fine PM
  cufftHandle plan_f_r2c = 0, plan_f_c2r = 0;
  float* rho_f = nullptr;       // padded real / complex in place
  float* force_f[3] = {nullptr, nullptr, nullptr};
  float* kern_f = nullptr;      // 3 planes of (nf/2+1)*nf*nf, scaled by 1/nf^3
  float* kern_f_raw = nullptr;  // unscaled copy kept only for inspection (may be null)
  // coarse PM
  cufftHandle plan_c_r2c = 0, plan_c_c2r = 0;
  float* rho_c = nullptr;
  float* force_c[3] = {nullptr, nullptr, nullptr};
  float* kern_c = nullptr;      // scaled by 1/nc^3 (exact: power of two)
  // PP
  float* fpp = nullptr;         // optional per-particle PP force (3*np), debug only
  // per-phase timers (null when disabled)
  struct CubeTimers* timers = nullptr;
  // stats
  DevStats* dstats = nullptr;
  DevStats* hstats = nullptr;   // pinned
  void* cufft_work = nullptr;
  size_t cufft_work_bytes = 0;
};

// ------------------------------------------------------------------ errors
int cube_fail(cube_ctx* c, int code, const std::string& msg);
#define CUBE_CUDA(ctx, call)                                                                   \
  do {                                                                                         \
    cudaError_t e_ = (call);                                                                   \
    if (e_ != cudaSuccess)                                                                     \
      return cube_fail(ctx, CUBE_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)
#define CUBE_FFT(ctx, call)                                                                    \
  do {                                                                                         \
    cufftResult r_ = (call);                                                                   \
    if (r_ != CUFFT_SUCCESS)                                                                   \
      return cube_fail(ctx, CUBE_ERR_CUDA, std::string(#call) + ": cufft error " + std::to_string((int)r_)); \
  } while (0)

// ------------------------------------------------------------- geometry
struct Geo {
  int nc, nt, nnt, ncell, ncb, nf;
  int izipx, izipv;
};
inline Geo make_geo(const cube_ctx* c) {
  Geo g;
  g.nc = c->p.nc;
  g.nt = c->nt;
  g.nnt = c->p.nnt;
  g.ncell = c->p.ncell;
  g.ncb = c->p.ncb;
  g.nf = c->nf;
  g.izipx = c->p.izipx;
  g.izipv = c->p.izipv;
  return g;
}

__host__ __device__ inline int wrapi(int a, int n) {
  int r = a % n;
  return r < 0 ? r + n : r;
}
// global coarse coordinates (0-based) -> cell id in the disjoint order
__host__ __device__ inline int64_t cell_id(const Geo& g, int gx, int gy, int gz) {
  int tx = gx / g.nt, ty = gy / g.nt, tz = gz / g.nt;
  int ix = gx - tx * g.nt, iy = gy - ty * g.nt, iz = gz - tz * g.nt;
  int64_t tile = tx + (int64_t)g.nnt * (ty + (int64_t)g.nnt * tz);
  return ix + (int64_t)g.nt * (iy + (int64_t)g.nt * (iz + (int64_t)g.nt * tile));
}
__host__ __device__ inline void cell_coords(const Geo& g, int64_t c, int& gx, int& gy, int& gz) {
  int64_t nt = g.nt;
  int ix = (int)(c % nt);
  c /= nt;
  int iy = (int)(c % nt);
  c /= nt;
  int iz = (int)(c % nt);
  c /= nt;
  int tx = (int)(c % g.nnt);
  c /= g.nnt;
  int ty = (int)(c % g.nnt);
  int tz = (int)(c / g.nnt);
  gx = tx * g.nt + ix;
  gy = ty * g.nt + iy;
  gz = tz * g.nt + iz;
}
// padded real-mesh index (row stride n+2), periodic in each dimension
__device__ __forceinline__ int64_t mesh_idx(int n, int x, int y, int z) {
  return (int64_t)x + (int64_t)(n + 2) * ((int64_t)y + (int64_t)n * z);
}

// ------------------------------------------------------- particle codes
__device__ __forceinline__ int load_code(const void* a, int64_t i, int nbytes) {
  return nbytes == 1 ? (int)((const int8_t*)a)[i] : (int)((const int16_t*)a)[i];
}
__device__ __forceinline__ void store_code(void* a, int64_t i, int nbytes, long long v) {
  if (nbytes == 1)
    ((int8_t*)a)[i] = (int8_t)(uint8_t)(unsigned long long)v;
  else
    ((int16_t*)a)[i] = (int16_t)(uint16_t)(unsigned long long)v;
}
// int(xp+ishift,izipx)+rshift == unsigned(xp)+0.5 (update_particle.f90:66)
__device__ __forceinline__ double pos_off(int code, int izipx) {
  int m = 1 << (8 * izipx);
  return (double)(code & (m - 1)) + 0.5;
}
__device__ __forceinline__ double xres_of(int izipx) { return izipx == 1 ? 1.0 / 256.0 : 1.0 / 65536.0; }

// tempx=ncell*(i-1)+ncell*(int+rshift)*x_resolution evaluated in real(8),
// rounded to real(4) (pm.f90:63); i is the tile-local 1-based cell index.
__device__ __forceinline__ float fine_tempx(int ncell, int ilocal, int code, int izipx) {
  double a = (double)(ncell * (ilocal - 1));
  double b = __dmul_rn(__dmul_rn((double)ncell, pos_off(code, izipx)), xres_of(izipx));
  return __double2float_rn(__dadd_rn(a, b));
}
// tempx=(i-1)+(int+rshift)*x_resolution-0.5 (pm.f90:221, 335)
__device__ __forceinline__ float coarse_tempx(int i1based, int code, int izipx) {
  double a = __dadd_rn((double)(i1based - 1), __dmul_rn(pos_off(code, izipx), xres_of(izipx)));
  return __double2float_rn(__dsub_rn(a, 0.5));
}

// sqrt(pi/2)/(sigma*vrel_boost) in real(8) (update_particle.f90:67)
inline double vcoef_host(float sigma);
__device__ __forceinline__ double vcoef(float sigma) {
  float s = __fsqrt_rn(__fdiv_rn(CUBE_PI_F, 2.0f));
  return __ddiv_rn((double)s, __dmul_rn((double)sigma, 2.5));
}
// vp=nint(real(nvbin-1)*atan(vcoef*v)/pi, kind=izipv) (update_particle.f90:117)
__device__ __forceinline__ long long v_encode(double v, double c, int nvbin) {
  double u = __ddiv_rn(__dmul_rn((double)(nvbin - 1), atan(__dmul_rn(c, v))), (double)CUBE_PI_F);
  return llround(u);
}
// one CIC kick term force*a_mid*dt/6/pi*wa*wb*wc in real(4), left to right (pm.f90:146)
__device__ __forceinline__ float kick_term(float f, float a_mid, float dt, float wa, float wb, float wc) {
  float r = __fmul_rn(f, a_mid);
  r = __fmul_rn(r, dt);
  r = __fdiv_rn(r, 6.0f);
  r = __fdiv_rn(r, CUBE_PI_F);
  r = __fmul_rn(r, wa);
  r = __fmul_rn(r, wb);
  return __fmul_rn(r, wc);
}

// host view of a float stored as its bit pattern
inline float bits_float(unsigned int u) {
  union {
    unsigned int i;
    float f;
  } x;
  x.i = u;
  return x.f;
}

// atomic max of a non-negative float via its bit pattern
__device__ __forceinline__ void atomic_max_pos(unsigned int* addr, float v) {
  atomicMax(addr, __float_as_uint(v));
}

// ----------------------------------------------------- host-side entry points
int cube_build_tables(cube_ctx* c);
int cube_ensure_decode(cube_ctx* c, double* tab, float sigma, float& cached);
int cube_kernels_init(cube_ctx* c, const float* fine_table, const float* coarse_table);
int cube_scan_counts(cube_ctx* c, const int32_t* counts, int64_t* starts, int64_t n);
int cube_update_x_impl(cube_ctx* c, float dt_old, float dt, float vz_max, cube_stats* st);
int cube_pp_impl(cube_ctx* c, float a_mid, float dt, cube_stats* st);
int cube_fine_density_impl(cube_ctx* c, cube_stats* st);
int cube_coarse_density_impl(cube_ctx* c, cube_stats* st);
int cube_fine_forces_impl(cube_ctx* c, cube_stats* st);
int cube_fine_kick_impl(cube_ctx* c, float a_mid, float dt);
int cube_coarse_forces_impl(cube_ctx* c, cube_stats* st);
int cube_coarse_kick_impl(cube_ctx* c, float a_mid, float dt, cube_stats* st);
int cube_state_in(cube_ctx* c, int64_t np, const void* xp, const void* vp, const int32_t* pid,
                  const int32_t* rhoc, const float* vfield);
int cube_state_out(cube_ctx* c, int64_t* np, void* xp, void* vp, int32_t* pid, int32_t* rhoc, float* vfield);
int cube_stats_fetch(cube_ctx* c);

// phase timers (cube_timing.cu); no-ops unless timing is enabled
enum {
  PH_UPD_DEST = 0, PH_UPD_RANK, PH_UPD_SCAN, PH_UPD_SCATTER, PH_UPD_SIGMA, PH_PP,
  PH_F_DEPOSIT, PH_F_R2C, PH_F_GREEN, PH_F_C2R, PH_F_F2MAX, PH_F_KICK,
  PH_C_DEPOSIT, PH_C_FFT, PH_C_KICK
};
void cube_phase_begin(cube_ctx* c, int phase);
void cube_phase_end(cube_ctx* c, int phase);
void cube_timers_free(cube_ctx* c);
struct PhaseScope {
  cube_ctx* c;
  int ph;
  PhaseScope(cube_ctx* cc, int p) : c(cc), ph(p) { cube_phase_begin(c, ph); }
  ~PhaseScope() { cube_phase_end(c, ph); }
};

// grid sizing: a multiple of the SM count
int cube_grid(int64_t work, int block, int max_blocks_per_sm = 16);
