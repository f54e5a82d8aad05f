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

#include <cmath>
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
  unsigned int ndense;           // destination cells left to the warp-per-cell vfield pass
  unsigned long long nexact;     // kick lanes evaluated on the exact FP64 chain
  unsigned int vmax_est_bits[3]; // fine kick: max |v + vfield| in FP32, when the last vmax is unknown
  double testrhof, testrhoc;
  unsigned long long rhof_fix, rhoc_fix;  // deposited mass in 2^-32 fixed point
  unsigned int pp_overflow;               // PP cells too dense for the global staging
  unsigned int nrank_dense;               // re-sort: source cells left to k_rank_dense
  unsigned int vmax_lo_bits[3];           // coarse kick: max of certified lower bounds of |v + vfield|
  unsigned long long pp_active;           // PP prefilter: particles with a neighbour besides themselves
};

// share of the last step's vmax above which the coarse kick evaluates a
// lane's |v + vfield| exactly (pm.f90:349)
constexpr float kVmaxTau = 0.95f;

// Scalars of one step when the step runs inside a captured CUDA graph
// (cube_batch_*).  A head kernel derives them on the device at the start of
// every step from the box's schedule and the previous step's results, with
// the eager host path's arithmetic; kernels read them through a StepDev
// pointer, null on the eager path, where the same values arrive as kernel
// arguments.
struct StepHost {
  float dt_mid, a_mid, dt;
  int nlayer;
  float tau[3];  // coarse kick: 0.7 of the last vmax
  float kick_f;  // PP kick factor a_mid*dt/6/pi, float and double
  double kick;
  float cf_vi;   // vcoef(sigma_vi) as float (the encode estimate only)
  int pad;
};
struct StepDev {
  StepHost h;
  float sigma_new, cf_new;  // update_x's sigma_vi_new and its vcoef
  // carried from step to step on the device
  float sigma_vi, vz_max;   // codec sigma of the state; sim%vz_max for nlayer
  float vmax_prev[3];       // the last coarse-kick vmax (0 before the first)
  int istep;                // steps done
};
// what the host reads back after a graph step: the stats of each stage
struct StepOut {
  DevStats upd, pp, fine, coarse;
  double sums[3];  // sigma statistics (update_particle.f90:171-224)
  float sigma_new;
  int pad;
};

struct cube_ctx {
  cube_params p{};
  int device = 0;
  cudaStream_t stream = nullptr;
  // a second particle species (the neutrinos of CUBEnu) shares the meshes,
  // FFT plans, force kernels and stream of the context it is linked to
  cube_ctx* owner = nullptr;
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
  uint8_t* doff = nullptr;      // cell offset source-destination of the primary copy, (dx+1)+3(dy+1)+9(dz+1); 255 if |d|>1
  uint16_t* lrank = nullptr;    // rank among the particles of one source cell bound for one destination
  uint16_t* offc = nullptr;     // 27 planes over the source cells: counts bound for each neighbour, then base ranks
  int32_t* perm = nullptr;      // new position -> old particle index
  int32_t* vdense = nullptr;    // destination cells with many particles (vfield_new by a warp each)
  uint32_t* rank = nullptr;     // rank of the primary copy in its destination
  int4* xtra = nullptr;         // extra copies: (particle, dest cell, rank, -)
  // general rank path: sort keys and entries (two buffers each, np_max +
  // xtra_cap) and the sort's scratch, allocated on first use
  uint64_t* skey[2] = {nullptr, nullptr};
  int32_t* sval[2] = {nullptr, nullptr};
  void* sort_tmp = nullptr;
  size_t sort_tmp_bytes = 0;
  int64_t xtra_cap = 0;
  void* scan_tmp = nullptr;
  size_t scan_tmp_bytes = 0;
  double* red_tmp = nullptr;    // block partial sums for sigma statistics
  int red_blocks = 0;
  // velocity code tables
  float* tan_tab = nullptr;     // float(tan(pi*v/(nvbin-1))) for v in [-nvbin/2, nvbin/2)
  struct Codec {
    float sigma = -1.f;
    double* dec = nullptr;     // dec[v+nvbin/2] = tan code / vcoef(sigma), real(8)
    float2* dech = nullptr;    // the same split into float hi + lo
    long long* bnd = nullptr;  // bnd[n] = bits of the smallest |v| that encodes to n (n=1..nvbin/2-1)
    int32_t* rt = nullptr;     // rt[v+nvbin/2] = the code of dec[v+nvbin/2] (a kick by zero)
  } codec[2];
  int codec_next = 0;
  float sigma_vi = 0.f, sigma_vi_new = 0.f;
  float vmax_prev[3] = {0.f, 0.f, 0.f};  // last coarse-kick vmax (0: unknown)
  // graph mode (cube_batch_*): step scalars on the device, codec slot 0 holds
  // sigma_vi and slot 1 sigma_vi_new, no host synchronisation inside a step
  bool graph_mode = false;
  StepDev* sd = nullptr;    // device
  StepOut* sout = nullptr;  // device (owned by the batch)
  unsigned long long kick_exact_lanes = 0;
  int opt_exact_kicks = 0;
  int opt_rank_walk = 0;   // ranks: 0 counting path (sort when it does not apply), 1 walker, 2 sort
  int rank_walked = 0;     // the last update used the walker
  int opt_pp_level = 0;  // first PP level (0-5)
  int opt_pp_heavy = 0;  // PP: entries from which a crowded block walks a particle with a warp (0: default)
  int opt_pp_parts = 0;  // PP: most parts a dense item is split into (0: default, 255)
  int opt_dep_fine = 0, opt_dep_coarse = 0;  // deposit brick shapes (0-3)
  int fail_alloc = 0;    // host fault injection: the n-th lazy allocation fails (0: off)
  cube_ctx* linked = nullptr;  // the second species linked to this context, if any
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
  float* fpp = nullptr;         // per-particle PP force (3*np_max): pair kernels -> kick pass
  int* pp_list[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};  // work of PP levels 1-5 (bricks, bricks, cells x3)
  int* pp_lpart[5] = {nullptr, nullptr, nullptr, nullptr, nullptr}; // their items' parts and claims
  float4* pp_scr_pts = nullptr;  // PP global staging (levels 4-5): pp_scr_cap float4, then 2 x pp_scr_cap uint32
  int64_t pp_scr_cap = 0;
  int* pp_nlist = nullptr;          // their lengths
  int* pp_nlist_host = nullptr;     // pinned copy of the last call's lengths
  int pp_brick_cap = 0;             // ceil(nc/4)^3
  // PP's prefilter (cube_pp.cu): a particle whose 27 neighbouring fine cells
  // hold no other particle has a zero pair force and a one-entry list; the
  // staging kernels then run over the other ("active") particles only
  unsigned long long* pp_occ = nullptr;  // 2 x ncells: occupied fine sub-cells, and those held twice or more
  unsigned* pp_act = nullptr;            // one bit per particle: active
  int32_t* pp_wcnt = nullptr;            // active particles per 32-particle word
  int64_t* pp_wstart = nullptr;          // their exclusive scan (words + 1)
  int32_t* pp_arhoc = nullptr;           // active particles per coarse cell
  int64_t* pp_acstart = nullptr;         // and their first position in pp_aidx
  int32_t* pp_aidx = nullptr;            // active particle indices, in storage order
  bool pp_act_valid = false;             // the last PP launch filtered: fpp holds the active particles only
  int opt_pp_filter = 0;                 // 0 automatic, 1 off, 2 on
  float pp_active_frac = 0.f;            // active share of the last filtered call (0: none yet)
  int pp_unfiltered = 0;                 // calls since the automatic choice last left the filter off
  // PP beside the PM force chain (cube_pp_particle_mesh): its own stream,
  // stats and pinned copy, and the fork / join events
  cudaStream_t stream_pp = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_pp = nullptr;
  DevStats* dstats_pp = nullptr;
  DevStats* hstats_pp = nullptr;  // pinned
  // host copies beside the step on their own stream: a download of xp, pid,
  // rhoc and vfield beside PP and PM, of vp beside the coarse kick
  // (cube_download_begin / _finish; calls that change the state are ordered
  // after it on the device by cube_copy_join), and an upload whose xp and vp
  // arrive in UP_PIECES pieces beside the re-sort's first pass and pid beside
  // the rest of the re-sort up to the scatter (cube_upload_begin; any other
  // call that reads the state first waits for all of it, cube_upload_join)
  static constexpr int UP_PIECES = 4;
  cudaStream_t stream_copy = nullptr;
  cudaEvent_t ev_copy_start = nullptr, ev_copy = nullptr, ev_pid = nullptr;
  cudaEvent_t ev_xv[UP_PIECES] = {};
  bool copy_pending = false;
  void* vp_host = nullptr;  // vp destination of a pending download
  bool pid_pending = false, xv_pending = false;
  int64_t up_np = 0;        // particle count of the pending upload's pieces
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
// Exact unsigned 32-bit division by a run-time constant with one high multiply
// (the round-up multiplier method of Granlund & Montgomery, 1994): 64-bit or
// generic integer division would go through the slow double-precision unit.
struct FastDiv {
  uint32_t d, m, s;
};
inline FastDiv make_fastdiv(uint32_t d) {
  FastDiv f{d, 0u, 0u};
  if (d <= 1) return f;
  uint32_t l = 0;
  while ((1ull << l) < d) l++;
  f.m = (uint32_t)((((1ull << l) - d) << 32) / d + 1);
  f.s = l;
  return f;
}
__host__ __device__ __forceinline__ uint32_t fdiv(uint32_t n, const FastDiv& f) {
  if (f.d <= 1) return n;
#ifdef __CUDA_ARCH__
  uint32_t t = __umulhi(n, f.m);
#else
  uint32_t t = (uint32_t)(((uint64_t)n * f.m) >> 32);
#endif
  return (t + ((n - t) >> 1)) >> (f.s - 1);
}

struct Geo {
  int nc, nt, nnt, ncell, ncb, nf;
  int izipx, izipv;
  FastDiv dnt, dnnt;  // division by nt and by nnt
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
  g.dnt = make_fastdiv((uint32_t)c->nt);
  g.dnnt = make_fastdiv((uint32_t)c->p.nnt);
  return g;
}

__host__ __device__ inline int wrapi(int a, int n) {
  int r = a % n;
  return r < 0 ? r + n : r;
}
// a in [-n, 2n): one compare instead of a division
__host__ __device__ __forceinline__ int wrap1(int a, int n) { return a < 0 ? a + n : (a >= n ? a - n : a); }
// global coarse coordinates (0-based) -> cell id in the disjoint order
__host__ __device__ inline int64_t cell_id(const Geo& g, int gx, int gy, int gz) {
  int tx = (int)fdiv((uint32_t)gx, g.dnt), ty = (int)fdiv((uint32_t)gy, g.dnt), tz = (int)fdiv((uint32_t)gz, g.dnt);
  int ix = gx - tx * g.nt, iy = gy - ty * g.nt, iz = gz - tz * g.nt;
  int tile = tx + g.nnt * (ty + g.nnt * tz);
  return (int64_t)(uint32_t)(ix + g.nt * (iy + g.nt * (iz + g.nt * tile)));
}
__host__ __device__ inline void cell_coords(const Geo& g, int64_t cid, int& gx, int& gy, int& gz) {
  uint32_t c = (uint32_t)cid, q;
  q = fdiv(c, g.dnt);
  int ix = (int)(c - q * (uint32_t)g.nt);
  c = q;
  q = fdiv(c, g.dnt);
  int iy = (int)(c - q * (uint32_t)g.nt);
  c = q;
  q = fdiv(c, g.dnt);
  int iz = (int)(c - q * (uint32_t)g.nt);
  c = q;
  q = fdiv(c, g.dnnt);
  int tx = (int)(c - q * (uint32_t)g.nnt);
  c = q;
  q = fdiv(c, g.dnnt);
  int ty = (int)(c - q * (uint32_t)g.nnt);
  int tz = (int)q;
  gx = tx * g.nt + ix;
  gy = ty * g.nt + iy;
  gz = tz * g.nt + iz;
}
// tile index and 1-based tile-local coordinate of a global coarse coordinate
__host__ __device__ __forceinline__ void tile_local(const Geo& g, int gc, int& T, int& L) {
  T = (int)fdiv((uint32_t)gc, g.dnt);
  L = gc - T * g.nt + 1;
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
// The real(8) sum is exact (< 28 significant bits), so one real(4) rounding
// of it equals one FP32 addition of the two exactly representable terms.
__device__ __forceinline__ float pos_off_f(int code, int izipx) {
  return (float)(code & ((1 << (8 * izipx)) - 1)) + 0.5f;
}
__device__ __forceinline__ float fine_tempx(int ncell, int ilocal, int code, int izipx) {
  float a = (float)(ncell * (ilocal - 1));
  float b = __fmul_rn(pos_off_f(code, izipx), izipx == 1 ? 4.0f / 256.0f : 4.0f / 65536.0f);
  return __fadd_rn(a, b);
}
// tempx=(i-1)+(int+rshift)*x_resolution-0.5 (pm.f90:221, 335)
__device__ __forceinline__ float coarse_tempx(int i1based, int code, int izipx) {
  float a = __fsub_rn((float)(i1based - 1), 0.5f);
  float b = __fmul_rn(pos_off_f(code, izipx), izipx == 1 ? 1.0f / 256.0f : 1.0f / 65536.0f);
  return __fadd_rn(a, b);
}

// sqrt(pi/2)/(sigma*vrel_boost) in real(8) (update_particle.f90:67)
inline double vcoef_host(float sigma) {
  volatile float s = std::sqrt(CUBE_PI_F / 2.0f);
  return (double)s / ((double)sigma * 2.5);
}
__device__ __forceinline__ double vcoef(float sigma) {
  float s = __fsqrt_rn(__fdiv_rn(CUBE_PI_F, 2.0f));
  return __ddiv_rn((double)s, __dmul_rn((double)sigma, 2.5));
}
// vp=nint(real(nvbin-1)*atan(vcoef*v)/pi, kind=izipv) (update_particle.f90:117)
__device__ __forceinline__ long long v_encode(double v, double c, int nvbin) {
  double u = __ddiv_rn(__dmul_rn((double)(nvbin - 1), atan(__dmul_rn(c, v))), (double)CUBE_PI_F);
  return llround(u);
}
// The same encode without FP64 transcendentals.  u(v) above is a monotone
// function of v and odd in v, so nint(u(v)) = sign(v) * #{n >= 1 : bnd[n] <= |v|},
// where bnd[n] is the smallest double whose u reaches n - 0.5 (found once per
// sigma by bisection over the doubles, k_encode_bounds).  An FP32 estimate
// picks the bin; at most a step or two of exact integer comparisons of the
// doubles' bit patterns (valid for non-negative doubles) settles it.
__device__ __forceinline__ float approx_float_pos(long long bits) {
  // truncate a non-negative double to float with integer operations only
  int e = (int)((bits >> 52) & 0x7ff) - 1023 + 127;
  if (e <= 0) return 0.f;
  if (e >= 255) return __int_as_float(0x7f800000);
  unsigned int m = (unsigned int)((bits >> 29) & 0x7fffff);
  return __int_as_float((e << 23) | m);
}
__device__ __forceinline__ long long v_encode_tab(double v, const long long* __restrict__ bnd, int nmax, float cf,
                                                  float amp) {
  long long bits = __double_as_longlong(v);
  long long ab = bits & 0x7fffffffffffffffLL;
  float af = approx_float_pos(ab);
  float u0 = amp * atanf(cf * af);
  int n = (int)(u0 + 0.5f);
  n = n < 0 ? 0 : (n > nmax ? nmax : n);
  while (n < nmax && __ldg(bnd + n + 1) <= ab) n++;
  while (n > 0 && __ldg(bnd + n) > ab) n--;
  return bits < 0 ? -(long long)n : (long long)n;
}
struct CodecView {
  const double* dec;
  const float2* dech;  // dec split into float hi + lo (hi = fl32(dec))
  const long long* bnd;
  int half, nmax;  // nvbin/2, nvbin/2-1
  float cf, amp;   // vcoef(sigma) and (nvbin-1)/pi as floats (estimate only)
  const float* cfp;  // when set, cf is read from the device (graph mode)
  const int32_t* rt;  // code of a zero kick: encode(decode(code)) (may be null)
};
__device__ __forceinline__ float codec_cf(const CodecView& k) { return k.cfp ? __ldg(k.cfp) : k.cf; }
__device__ __forceinline__ double codec_decode(const CodecView& k, int code) { return __ldg(k.dec + code + k.half); }
__device__ __forceinline__ float2 codec_decode_ff(const CodecView& k, int code) {
  return __ldg(k.dech + code + k.half);
}
__device__ __forceinline__ long long codec_encode(const CodecView& k, double v) {
  return v_encode_tab(v, k.bnd, k.nmax, codec_cf(k), k.amp);
}

// ---------------------------------------------------------------------------
// FP64-free fast paths.  GB300 issues about one FP64 instruction per SM clock
// (1/128 of FP32), so the hot loops evaluate the reference's FP64 expressions
// in FP32 / float-float with a rigorous error bound, and keep the result only
// when every real number inside the bound gives the same integer or float;
// otherwise the lane evaluates the reference's FP64 expression itself.  The
// stored result is therefore the reference's bit for bit.
constexpr float kU24 = 5.9604645e-8f;  // 2^-24

// exact float -> double bit pattern with integer operations (subnormals -> +-0)
__device__ __forceinline__ long long f2d_bits(float f) {
  unsigned int u = __float_as_uint(f);
  unsigned int ex = (u >> 23) & 0xffu;
  unsigned long long s = (unsigned long long)(u >> 31) << 63;
  if (ex == 0u) return (long long)s;
  unsigned long long e64 = ex == 0xffu ? 0x7ffull : (unsigned long long)(ex - 127u + 1023u);
  return (long long)(s | (e64 << 52) | ((unsigned long long)(u & 0x7fffffu) << 29));
}

// The velocity code of any |V| in [ab - E, ab + E] (ab = bit pattern of a
// non-negative double, E >= 0) is n: returns true and n when the whole
// interval lies in one code bin.  Distances are counted in ulps of ab's binade;
// an edge in another binade is at least as far as that binade's end.
// the three parts of certify_abs: the FP32 estimate of the bin, the probe of
// its two edges, and the check on the edges the probe (or a walk) found
__device__ __forceinline__ long long certify_estimate(long long ab, const CodecView& k) {
  float af = approx_float_pos(ab);
  float u0 = k.amp * atanf(codec_cf(k) * af);
  int m = (int)(u0 + 0.5f);
  return m < 0 ? 0 : (m > k.nmax ? k.nmax : m);
}
__device__ __forceinline__ void certify_probe(long long n, const CodecView& k, long long& lb, long long& ub) {
  lb = n > 0 ? __ldg(k.bnd + n) : 0;
  ub = n < k.nmax ? __ldg(k.bnd + n + 1) : 0x7fffffffffffffffLL;
}
__device__ __forceinline__ bool certify_finish(long long ab, float E, const CodecView& k, long long n, long long lb,
                                               long long ub, long long* n_out) {
  if (ab < lb || ab >= ub) {
    while (n < k.nmax && __ldg(k.bnd + n + 1) <= ab) n++;
    while (n > 0 && __ldg(k.bnd + n) > ab) n--;
    certify_probe(n, k, lb, ub);
  }
  *n_out = n;
  int e = (int)((ab >> 52) & 0x7ff);
  if (e == 0 || e >= 0x7fe) return n == 0 && e == 0;  // subnormal |V| is deep inside code 0
  int sh = 1075 - e;                                   // E in ulps of this binade: E * 2^sh
  float kf = (sh >= -126 && sh <= 127) ? __fmul_rn(E, __int_as_float((127 + sh) << 23)) : ldexpf(E, sh);
  if (!(kf < 4.0e15f)) return false;
  long long kk = (kf < 2147483648.0f ? (long long)(unsigned int)kf : (long long)kf) + 1;
  long long blo = (long long)e << 52, bhi = (long long)(e + 1) << 52;
  if (n > 0) {
    long long lx = lb > blo ? lb : blo;
    if (ab - lx <= kk) return false;
  }
  if (n < k.nmax) {
    long long ux = ub < bhi ? ub : bhi;
    if (ux - ab <= kk) return false;
  }
  return true;
}
__device__ __forceinline__ bool certify_abs(long long ab, float E, const CodecView& k, long long* n_out) {
  // the FP32 estimate is within a few hundredths of a code: probe its bin with
  // two independent loads, walk only when it fell on the wrong side of an edge
  const long long n = certify_estimate(ab, k);
  long long lb, ub;
  certify_probe(n, k, lb, ub);
  return certify_finish(ab, E, k, n, lb, ub, n_out);
}
// certify_abs of three values with the table probes of all three issued
// together, so no value's loads wait for another's
__device__ __forceinline__ void certify_abs3(const long long ab[3], const float E[3], const CodecView& k,
                                             long long n_out[3], bool ok[3]) {
  long long n[3], lb[3], ub[3];
#pragma unroll
  for (int d = 0; d < 3; d++) n[d] = certify_estimate(ab[d], k);
#pragma unroll
  for (int d = 0; d < 3; d++) certify_probe(n[d], k, lb[d], ub[d]);
#pragma unroll
  for (int d = 0; d < 3; d++) ok[d] = certify_finish(ab[d], E[d], k, n[d], lb[d], ub[d], &n_out[d]);
}

__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// vreal=vreal+f_tot*a_mid*dt/6/pi in FP64 and its code (ext_pp_force.f90:
// 116-121), for lanes the fast tiers leave undecided (not inlined: keeps
// double conversions off the common path)
static __device__ __noinline__ long long pp_kick_exact(CodecView cv, int code, float F, double kick) {
  double v = __dadd_rn(codec_decode(cv, code), __dmul_rn((double)F, kick));
  return codec_encode(cv, v);
}

// The PP kick of one particle's three velocity codes: v = decode(code) +
// F*kick, encoded with the same sigma.  The FP32 sum of the decode's float
// hi and the FP32 kick product is certified against its bound (the
// product's two roundings, the hi split and the sum's rounding) with the
// three table probes issued together; undecided lanes take the FP64
// expression.  code[] is updated in place.
__device__ __forceinline__ void pp_kick3(const CodecView& cv, int code[3], const float F[3], float kick_f,
                                         double kick_d, int exact_only) {
  float E[3], vf[3];
  long long ab[3], n[3];
  bool ok[3];
#pragma unroll
  for (int d = 0; d < 3; d++) {
    const float dh = codec_decode_ff(cv, code[d]).x;
    const float kf = __fmul_rn(F[d], kick_f);
    vf[d] = __fadd_rn(dh, kf);
    E[d] = 1.25f * (fabsf(kf) * 1.3e-7f + (2.f * fabsf(dh) + fabsf(vf[d])) * 6.0e-8f);
    ab[d] = f2d_bits(vf[d]) & 0x7fffffffffffffffLL;
  }
  certify_abs3(ab, E, cv, n, ok);
#pragma unroll
  for (int d = 0; d < 3; d++)
    code[d] = (!exact_only && ok[d]) ? (int)(vf[d] < 0.f ? -n[d] : n[d])
                                     : (int)pp_kick_exact(cv, code[d], F[d], kick_d);
}

// Nearest float to the real t + lo, certified when every real within margin
// of it rounds to the same float: its distance from rr stays below half an ulp
// (a quarter ulp when rr is a power of two, where the spacing below halves).
// diff carries one FP32 rounding, covered by the 2^-20 inflation.
__device__ __forceinline__ bool round_certified(float t, float lo, float margin, float* r) {
  float rr = __fadd_rn(t, lo);
  float diff = __fadd_rn(__fsub_rn(t, rr), lo);
  unsigned int u = __float_as_uint(rr), e = (u >> 23) & 0xffu;
  *r = rr;
  if (e <= 25u || e == 0xffu) return false;
  float quarter_ulp = __uint_as_float((e - 25u) << 23);
  float lim = (u & 0x7fffffu) == 0u ? quarter_ulp : 2.0f * quarter_ulp;
  return fabsf(diff) * 1.000001f + margin < lim;
}

// nint(x) of the reference (halves away from zero) for every x within E of xf
__device__ __forceinline__ bool nint_certified(float xf, float E, long long* out) {
  float a = fabsf(xf);
  E = E * 1.01f + (a + 1.0f) * 2.4e-7f;  // cover the FP32 roundings of the test below
  float lo = floorf(__fadd_rn(__fsub_rn(a, E), 0.5f)), hi = floorf(__fadd_rn(__fadd_rn(a, E), 0.5f));
  if (lo != hi || !(a < 1.0e9f)) return false;
  long long r = (long long)hi;
  *out = xf < 0.f ? -r : r;
  return true;
}

// x/c correctly rounded, for a constant c with rc = RN(1/c): q = RN(x*rc), the
// residual x - q*c is exact in one FMA, and q + residual*rc rounds to RN(x/c)
// (Markstein's correction step, IBM J. Res. Dev. 34(1), 1990).  For c = 6 and
// c = pi_f the identity with __fdiv_rn is checked for every float by
// cube_arith_check; zeros keep their sign through the product, tiny, huge and
// non-finite x take the IEEE division.
constexpr float kDivLo = 7.888609052210118e-31f;  // 2^-100
constexpr float kDivHi = 1.2676506002282294e30f;  // 2^100
__device__ __forceinline__ float div_const(float x, float c, float rc) {
  float ax = fabsf(x);
  if (ax == 0.f) return __fmul_rn(x, rc);
  if (!(ax >= kDivLo && ax <= kDivHi)) return __fdiv_rn(x, c);
  float q = __fmul_rn(x, rc);
  float r = __fmaf_rn(-q, c, x);
  return __fmaf_rn(r, rc, q);
}

// one CIC kick term force*a_mid*dt/6/pi*wa*wb*wc in real(4), left to right
// (pm.f90:146), split at the weights: kick_pre depends on the mesh point only,
// kick_w applies the particle's three CIC weights to it
__device__ __forceinline__ float kick_pre(float f, float a_mid, float dt) {
  float r = __fmul_rn(f, a_mid);
  r = __fmul_rn(r, dt);
  r = div_const(r, 6.0f, 0.16666667163372040f);         // RN(1/6)
  return div_const(r, CUBE_PI_F, 0.31830987334251404f);  // RN(1/pi_f)
}
__device__ __forceinline__ float kick_w(float g, float wa, float wb, float wc) {
  return __fmul_rn(__fmul_rn(__fmul_rn(g, wa), wb), wc);
}
__device__ __forceinline__ float kick_term(float f, float a_mid, float dt, float wa, float wb, float wc) {
  return kick_w(kick_pre(f, a_mid, dt), wa, wb, wc);
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

// ------------------------------------------------------- block helpers
// In-place exclusive scan of n ints by the whole block (blockDim.x a multiple
// of 32, at most 1024); returns the total to every thread.  Each thread scans a
// contiguous run, the run sums are scanned across warps.  Ends with a barrier.
__device__ __forceinline__ int block_exclusive_scan(int* v, int n) {
  __shared__ int wsum[32];
  const int t = threadIdx.x, lane = t & 31, w = t >> 5, nw = blockDim.x >> 5;
  const int per = (n + blockDim.x - 1) / blockDim.x;
  const int b0 = min(n, t * per), b1 = min(n, b0 + per);
  int s = 0;
  for (int i = b0; i < b1; i++) s += v[i];
  int inc = s;
  for (int o = 1; o < 32; o <<= 1) {
    int y = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += y;
  }
  if (lane == 31) wsum[w] = inc;
  __syncthreads();
  int wbase = 0, total = 0;
  for (int k = 0; k < nw; k++) {
    int x = wsum[k];
    if (k < w) wbase += x;
    total += x;
  }
  int run = wbase + inc - s;
  for (int i = b0; i < b1; i++) {
    int x = v[i];
    v[i] = run;
    run += x;
  }
  __syncthreads();
  return total;
}

// The same for n 16-bit counts whose total stays below 65536.
__device__ __forceinline__ int block_exclusive_scan_u16(unsigned short* v, int n) {
  __shared__ int wsum16[32];
  const int t = threadIdx.x, lane = t & 31, w = t >> 5, nw = blockDim.x >> 5;
  const int per = (n + blockDim.x - 1) / blockDim.x;
  const int b0 = min(n, t * per), b1 = min(n, b0 + per);
  int s = 0;
  for (int i = b0; i < b1; i++) s += v[i];
  int inc = s;
  for (int o = 1; o < 32; o <<= 1) {
    int y = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += y;
  }
  if (lane == 31) wsum16[w] = inc;
  __syncthreads();
  int wbase = 0, total = 0;
  for (int k = 0; k < nw; k++) {
    int x = wsum16[k];
    if (k < w) wbase += x;
    total += x;
  }
  int run = wbase + inc - s;
  for (int i = b0; i < b1; i++) {
    int x = v[i];
    v[i] = (unsigned short)run;
    run += x;
  }
  __syncthreads();
  return total;
}

// Visit every particle of a box of source cells: cell t = sx + S0*row has
// pref[t] particles before it (exclusive scan over the box, pref[ns] not
// needed) and its first particle at sstart[t].  One warp per row of S0 <= S0MAX
// cells along x: the row's particles are consecutive in j, and the cell of
// each j is found by comparing with the row's prefix values held in registers.
// f(p, sx, row) is called once per particle (p its storage index).
template <int S0MAX, class F>
__device__ __forceinline__ void for_box_particles(const int* pref, const long long* sstart, int S0, int nrows,
                                                  int total, F&& f) {
  const int lane = threadIdx.x & 31;
  for (int row = threadIdx.x >> 5; row < nrows; row += blockDim.x >> 5) {
    const int t0 = row * S0;
    int rp[S0MAX];
#pragma unroll
    for (int q = 0; q < S0MAX; q++) rp[q] = q < S0 ? pref[t0 + q] : 0x7fffffff;
    const int jend = row + 1 < nrows ? pref[t0 + S0] : total;
    for (int j = rp[0] + lane; j < jend; j += 32) {
      int cs = rp[0], sx = 0;
#pragma unroll
      for (int q = 1; q < S0MAX; q++)
        if (rp[q] <= j) {
          cs = rp[q];
          sx = q;
        }
      f((int64_t)(sstart[t0 + sx] + (j - cs)), sx, row);
    }
  }
}

// ----------------------------------------------------- host-side entry points
int cube_build_tables(cube_ctx* c);
// decode/encode tables for up to two sigma values at once (built on demand)
int cube_codec_pair(cube_ctx* c, float s1, float s2, CodecView* v1, CodecView* v2);
// graph mode: tables of a slot from a device sigma; a view reading cf from the device
int cube_codec_build_dev(cube_ctx* c, int slot, const float* sigp);
void cube_codec_view_dev(const cube_ctx* c, int slot, const float* cfp, CodecView* v);
int cube_kernels_init(cube_ctx* c, const float* fine_table, const float* coarse_table);
int cube_scan_counts(cube_ctx* c, const int32_t* counts, int64_t* starts, int64_t n);
int cube_update_x_impl(cube_ctx* c, float dt_old, float dt, float vz_max, cube_stats* st);
int cube_pp_impl(cube_ctx* c, float a_mid, float dt, cube_stats* st);
// defer_kick: leave the kick to the fine kick (cube_fine_kick_impl with_pp)
int cube_pp_launch(cube_ctx* c, float a_mid, float dt, bool defer_kick = false);
int cube_pp_init(cube_ctx* c);  // once per context: the staging kernels' shared-memory sizes
int cube_pp_finish(cube_ctx* c, cube_stats* st);
// density deposits; accumulate: add to the mesh (the linked species) instead of writing it
int cube_fine_density_impl(cube_ctx* c, cube_stats* st, bool accumulate = false);
int cube_coarse_density_impl(cube_ctx* c, cube_stats* st, bool accumulate = false);
// pre (a_mid, dt) non-null: after the maxima, the force meshes are rewritten
// as the mesh part of the kick term, force*a_mid*dt/6/pi, and the kick that
// follows is given pre=true (fused step only; the stage calls keep forces)
int cube_fine_forces_impl(cube_ctx* c, cube_stats* st, const float* pre = nullptr);
// with_pp: first apply the PP kick that cube_pp_launch(.., defer_kick) left
// to the fine kick (eager mode)
int cube_fine_kick_impl(cube_ctx* c, float a_mid, float dt, bool pre = false, bool with_pp = false);
int cube_coarse_forces_impl(cube_ctx* c, cube_stats* st, const float* pre = nullptr);
int cube_coarse_kick_impl(cube_ctx* c, float a_mid, float dt, cube_stats* st, bool pre = false);
int cube_fine_spectral_impl(cube_ctx* c, cube_stats* st, const float* pre);
int cube_coarse_spectral_impl(cube_ctx* c, cube_stats* st, const float* pre);
int cube_pk_deposit(cube_ctx* c, int ng, float* rho, unsigned long long* total);
int dep_shift(float mass);  // deposits' fixed point: total = integer * 2^-dep_shift(mass)
// initial-condition pieces shared with the differentiable form (cube_ic.cu):
// the real filter noise -> phi on an n^3 lattice (Delta^2 scaling times the
// corrected potential kernel, 1/n^3 folded in), the counter-hash noise, and a^2 H
int cube_ic_filter(cube_ctx* c, const cube_cosmology& cs, double a, int n, cufftHandle r2c, cufftHandle c2r,
                   float* scratch, float* dtab, float* filter);
void cube_ic_noise(float* r, int n, int pitch, uint32_t seed, cudaStream_t s);
double cube_ic_vfactor(double a, double om, double ol);
int cube_state_in(cube_ctx* c, int64_t np, const void* xp, const void* vp, const int32_t* pid,
                  const int32_t* rhoc, const float* vfield, bool defer_pid = false);
int cube_state_out(cube_ctx* c, int64_t* np, void* xp, void* vp, int32_t* pid, int32_t* rhoc, float* vfield);
// orders the context stream after a pending cube_download_begin copy
int cube_copy_join(cube_ctx* c);
// stable radix sort of n (key, entry) pairs over key bits [begin_bit, end_bit)
// from skey[0]/sval[0]; *keys, *vals receive the buffers holding the result
int cube_sort_pairs(cube_ctx* c, int64_t n, int begin_bit, int end_bit, uint64_t** keys, int32_t** vals);
// orders the context stream after a deferred pid upload
int cube_pid_join(cube_ctx* c);
// ... after every piece of a pending cube_upload_begin (xp, vp and pid)
int cube_upload_join(cube_ctx* c);
int cube_copy_stream(cube_ctx* c);
int cube_state_out_begin(cube_ctx* c, int64_t* np, void* xp, void* vp, int32_t* pid, int32_t* rhoc, float* vfield);
int cube_state_out_finish(cube_ctx* c);
int cube_stats_fetch(cube_ctx* c);

// phase timers (cube_timing.cu); no-ops unless timing is enabled
enum {
  PH_UPD_DEST = 0, PH_UPD_RANK, PH_UPD_SCAN, PH_UPD_SCATTER, PH_UPD_SIGMA, PH_PP,
  PH_F_DEPOSIT, PH_F_R2C, PH_F_GREEN, PH_F_C2R, PH_F_F2MAX, PH_F_KICK,
  PH_C_DEPOSIT, PH_C_FFT, PH_C_KICK, PH_UPD_PLACE
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
