// cube_pp.cu -- ext_pp_force (ext_pp_force.f90:10-162) on GB300.
//
// The reference threads a linked list through the fine cells of each tile
// (hoc/ll, ext_pp_force.f90:53-75) and, for every particle of a physical fine
// cell, sums m*r/|r|^3*pcut(|r|) over the particles of the 3^3 neighbouring
// fine cells, skipping pairs with |r| <= rsoft (:94-110), in FP64.
//
// Here a block of coarse cells is staged in shared memory: the particles of
// the block and of the one-fine-cell layer around it, read from the block's
// cells and its ring of coarse cells (storage is ordered by coarse cell), as
// FP32 positions relative to the block (exact: 4*frac has at most 17 bits),
// then counting-sorted by fine cell, each fine cell's particles by index, so
// each particle of the block walks exactly its 27 neighbouring fine cells, as
// the linked list does.  Pair forces are FP32, summed with compensation
// (Kahan) in that fixed order: bitwise reproducible whichever kernel handles
// a particle, within about one rounding of the exact sum of the FP32 terms.
//
// Six levels keep dense regions correct without a host round trip; each
// level lists what did not fit for the next one:
//   0. one block per brick of 4^3 coarse cells, 1536 staged particles at most
//      (several blocks per SM; a uniform brick stages about 1100);
//   1. listed bricks again, one 1024-thread block per SM with 8960 of room;
//   2. the cells of bricks listed by level 1, one at a time, 1536 of room;
//   3. listed cells with 8960 of room;
//   4. listed cells staged in a global scratch, an equal region per block;
//   5. the rest, one block with the whole scratch (2^22 entries at most; a
//      cell beyond that is reported as a PP overflow, ext_pp_force.f90:41-45).
// A crowded block walks its particles in fine-cell order, so the lanes of a
// warp share their neighbour bins (at z = 0 this took PP from 59 to 24 ms
// for 256^3 particles).
// The kick (a pass of its own over the particles in storage order, from the
// per-particle sums the pair kernels leave) adds F*a_mid*dt/(6 pi) in FP64 as
// one product with the precomputed factor -- the FP32 pair sum already sets
// this kick's tolerance against the reference's FP64 sum -- and the velocity
// code is the exact code of
// update_particle.f90:117 (certified FP32 fast path, FP64 when ambiguous).
#include <algorithm>
#include <cmath>

#include "cube_internal.cuh"

namespace {

constexpr int PB = 4;                          // coarse cells per brick edge
constexpr int PS_MAX = PB + 2;                 // staged coarse cells per edge
constexpr int PNS_MAX = PS_MAX * PS_MAX * PS_MAX;
constexpr int PNCORE_MAX = PB * PB * PB;
constexpr int PNF_MAX = (4 * PB + 2) * (4 * PB + 2) * (4 * PB + 2);
constexpr int PNROW_MAX = (4 * PB) * (4 * PB);  // core rows of fine cells in a brick
constexpr int PP_CAP = 1536;      // staged particles per brick (several blocks per SM)
constexpr int PP_CAP1 = 8960;     // staged particles per single cell (one block per SM)
constexpr int PP_THREADS = 256;
constexpr int PP_THREADS1 = 1024;
constexpr int PNF1 = 6 * 6 * 6;   // staged fine cells of one coarse cell and its ring
// shared memory of one block: staged points, bin/rank words, slots by bin, 16-bit bin offsets
constexpr size_t pp_smem(int cap, int nf) {
  return (sizeof(float4) + sizeof(unsigned) + sizeof(unsigned short)) * (size_t)cap +
         sizeof(unsigned short) * (size_t)(nf + 2);
}
constexpr size_t PP_SMEM = pp_smem(PP_CAP, PNF_MAX);
constexpr size_t PP_SMEM1 = pp_smem(PP_CAP1, PNF1);
constexpr size_t PP_SMEM1B = pp_smem(PP_CAP1, PNF_MAX);
// level 0 when few particles are staged (the prefilter on a sparse state):
// 384 staged particles in 128-thread blocks, eight blocks per SM instead of
// four, more bricks in flight to hide the staging's latency
constexpr int PP_CAP_S = 384;
constexpr int PP_THREADS_S = 128;
constexpr size_t PP_SMEM_S = pp_smem(PP_CAP_S, PNF_MAX);
constexpr float PP_SPARSE_FRAC = 0.25f;  // active share below which level 0 takes the small blocks
static_assert(PP_CAP1 < 65536 && PP_CAP1 < (1 << 19), "slots are 16-bit, ranks fit 19 bits");
static_assert(PNF_MAX < (1 << 13) && PNF1 < (1 << 8), "bins fit 13 bits (bricks) and 8 bits (cells)");

struct PPArgs {
  Geo g;
  int64_t np;
  const void* xp;
  void* vp;
  const int32_t* rhoc;
  const int64_t* cstart;
  CodecView cv;
  float mass, rsoft, inv_cut;
  double kick;   // a_mid*dt/6/pi
  float kick_f;  // the same rounded to float (fast path)
  int exact_only;
  int heavy;     // entries from which a crowded block walks a particle with a warp
  int max_parts; // most parts a dense item is split into
  float* fpp;    // per-particle summed pair force (3 per particle), pair kernels -> kick pass
  int nb;        // bricks per dimension
  int* list[5];    // work of levels 1..5: bricks, bricks, cells, cells, cells
  int* lpart[5];   // per listed item: parts (low 8 bits), parts claimed (above)
  int* nlist;      // their lengths (5), then each level's next-item counter (6)
  float4* scr_pts;     // global staging of levels 4-5 (scr_cap entries each)
  unsigned* scr_kinfo;
  unsigned* scr_order;
  int64_t scr_cap;
  DevStats* st;
  const StepDev* sd;  // graph mode: the kick factors from the device
  const int32_t* pidx;  // prefilter: staged positions -> particle index (null: the identity)
  const unsigned* act;  // prefilter: one bit per particle, set where fpp was written (null: all)
  const int64_t* nact;  // prefilter: the number of active particles (the entries of pidx)
};
__device__ __forceinline__ float pp_kick_f(const PPArgs& a) { return a.sd ? __ldg(&a.sd->h.kick_f) : a.kick_f; }
__device__ __forceinline__ double pp_kick_d(const PPArgs& a) { return a.sd ? __ldg(&a.sd->h.kick) : a.kick; }

__device__ __forceinline__ float fine_off(int code, int izipx) {
  // ncell*(int(xp+ishift)+rshift)*x_resolution: exact in real(4)
  return __fmul_rn(pos_off_f(code, izipx), izipx == 1 ? 4.0f / 256.0f : 4.0f / 65536.0f);
}

// Compensated (Kahan) FP32 summation: the sum of a particle's pair forces,
// taken in one fixed order (its 27 neighbouring fine cells row by row, each
// fine cell's particles by increasing index), so every level and every run
// gives the same bits; the compensation keeps the sum within about one
// rounding of the exact sum of the FP32 pair forces.
__device__ __forceinline__ void kahan_add(float& sum, float& comp, float x) {
  const float y = __fsub_rn(x, comp);
  const float t = __fadd_rn(sum, y);
  comp = __fsub_rn(__fsub_rn(t, sum), y);
  sum = t;
}

// v*2^32 as a two's-complement int64 from 32-bit conversions only (|v| < 2^23;
// truncated toward zero)
__device__ __forceinline__ long long to_fix(float v) {
  float a = fabsf(v);
  float ws = __fmul_rn(a, 256.0f), fh = floorf(ws);
  long long q = ((long long)(unsigned int)fh << 24) + (unsigned int)__fmul_rn(__fsub_rn(ws, fh), 16777216.0f);
  return v < 0.f ? -q : q;
}
__device__ __forceinline__ float from_fix(long long q) {
  bool neg = q < 0;
  unsigned long long u = neg ? (unsigned long long)(-q) : (unsigned long long)q;
  float hi = (float)(unsigned int)(u >> 32), lo = (float)(unsigned int)(u & 0xffffffffull);
  float r = __fmaf_rn(lo, 2.3283064365386963e-10f, hi);
  return neg ? -r : r;
}

// A particle's neighbour list (27 fine cells, 9 row ranges, particles by
// index) is summed in chunks of PP_CHUNK consecutive entries: each chunk's
// pair forces in a compensated sum from zero, the chunks' values (sum minus
// compensation) added in 2^-32 fixed point, exactly and in any order.  A
// thread walking the whole list and a warp whose lanes take one chunk each
// therefore give the same bits.
constexpr int PP_CHUNK = 32;
// entries from which a crowded block's particle is walked by a warp: only
// extreme lists (parts already spread dense items over SMs, and the warp
// walk's own overhead made 1024 and 256 slower at z = 0)
constexpr int PP_HEAVY = 8192;
constexpr int PP_HEAVY_LIST = 256;  // heavy particles a block lists (more: the warp walk scans the part)

__device__ __forceinline__ void pp_fold(long long* Q, float* s, float* c) {
#pragma unroll
  for (int d = 0; d < 3; d++) {
    Q[d] += to_fix(__fsub_rn(s[d], c[d]));
    s[d] = c[d] = 0.f;
  }
}

// one pair: add the force of a particle at offset r (FP32).  1/|r| is the
// correctly rounded reciprocal square root, |r| = r^2 * (1/|r|), and 1/|r|^3
// three more roundings: within about two ulps like the square root plus
// division it replaces, at fewer instructions (the approximate hardware
// reciprocal square root alone moved the codes of the strongest kicks by two)
__device__ __forceinline__ void pair_force(const PPArgs& a, float rx, float ry, float rz, float* sum, float* comp) {
  // explicit roundings: every kernel evaluates the same bits for a pair
  float r2 = __fmaf_rn(rx, rx, __fmaf_rn(ry, ry, __fmul_rn(rz, rz)));
  float ri = __frsqrt_rn(r2);    // +inf for the self pair
  float rm = __fmul_rn(r2, ri);  // NaN for the self pair
  if (!(rm > a.rsoft)) return;   // merge(force,0,rmag>rsoft); self pairs excluded
  float rc = __fmul_rn(rm, a.inv_cut);
  float rc3 = __fmul_rn(__fmul_rn(rc, rc), rc);
  // pcut = 1 - 1.75 rc^3 + 0.75 rc^5  (ext_pp_force.f90:107)
  float pcut = __fmaf_rn(__fmul_rn(0.75f, rc3), __fmul_rn(rc, rc), __fmaf_rn(-1.75f, rc3, 1.0f));
  float s = __fmul_rn(__fmul_rn(a.mass, pcut), __fmul_rn(__fmul_rn(ri, ri), ri));
  kahan_add(sum[0], comp[0], __fmul_rn(s, rx));
  kahan_add(sum[1], comp[1], __fmul_rn(s, ry));
  kahan_add(sum[2], comp[2], __fmul_rn(s, rz));
}

// the summed pair force of particle p, kept for the kick pass; returns |F|^2
__device__ __forceinline__ float pp_store_force(const PPArgs& a, int64_t p, const long long* Q) {
  float F[3];
  for (int d = 0; d < 3; d++) {
    F[d] = from_fix(Q[d]);
    a.fpp[3 * p + d] = F[d];
  }
  return __fmaf_rn(F[0], F[0], __fmaf_rn(F[1], F[1], __fmul_rn(F[2], F[2])));
}

// kick + exact velocity code of every particle, in storage order (coalesced
// code and force accesses; the pair kernels visit particles in staging order)
__global__ void __launch_bounds__(256) k_pp_kick(PPArgs a) {
  const Geo& g = a.g;
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < a.np; p += (int64_t)gridDim.x * blockDim.x) {
    float F[3];
    int code[3];
    // a particle the prefilter left out has a zero pair force (fpp not written)
    const bool on = !a.act || ((__ldg(a.act + (p >> 5)) >> (p & 31)) & 1u);
#pragma unroll
    for (int d = 0; d < 3; d++) {
      F[d] = on ? a.fpp[3 * p + d] : 0.f;
      code[d] = load_code(a.vp, 3 * p + d, g.izipv);
    }
    pp_kick3(a.cv, code, F, pp_kick_f(a), pp_kick_d(a), a.exact_only);
#pragma unroll
    for (int d = 0; d < 3; d++) store_code(a.vp, 3 * p + d, g.izipv, code[d]);
  }
}

// With the prefilter: the kick of the active particles (the list pidx) ...
__global__ void __launch_bounds__(256) k_pp_kick_active(PPArgs a) {
  const Geo& g = a.g;
  const int64_t n = __ldg(a.nact);
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t p = __ldg(a.pidx + i);
    float F[3];
    int code[3];
#pragma unroll
    for (int d = 0; d < 3; d++) {
      F[d] = a.fpp[3 * p + d];
      code[d] = load_code(a.vp, 3 * p + d, g.izipv);
    }
    pp_kick3(a.cv, code, F, pp_kick_f(a), pp_kick_d(a), a.exact_only);
#pragma unroll
    for (int d = 0; d < 3; d++) store_code(a.vp, 3 * p + d, g.izipv, code[d]);
  }
}
// ... and of the others: a zero force, so each code becomes the code of its
// own decoded value (the codec's zero-kick table)
__global__ void __launch_bounds__(256) k_pp_kick_idle(PPArgs a) {
  const Geo& g = a.g;
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < a.np; p += (int64_t)gridDim.x * blockDim.x) {
    if ((__ldg(a.act + (p >> 5)) >> (p & 31)) & 1u) continue;
#pragma unroll
    for (int d = 0; d < 3; d++)
      store_code(a.vp, 3 * p + d, g.izipv, __ldg(a.cv.rt + load_code(a.vp, 3 * p + d, g.izipv) + a.cv.half));
  }
}

__device__ __forceinline__ void pp_reduce(const PPArgs& a, unsigned long long npairs, unsigned long long nwork,
                                          float f2max) {
  for (int o = 16; o > 0; o >>= 1) {
    npairs += __shfl_xor_sync(0xffffffffu, npairs, o);
    nwork += __shfl_xor_sync(0xffffffffu, nwork, o);
    f2max = fmaxf(f2max, __shfl_xor_sync(0xffffffffu, f2max, o));
  }
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(&a.st->npairs, npairs);
    atomicAdd(&a.st->itest1, nwork);
    atomic_max_pos(&a.st->f2_pp_bits, f2max);
  }
}

struct PPSmem {
  int pref[PNS_MAX + 1];         // ring-and-block particles before each staged cell
  long long sstart[PNS_MAX];     // first particle of each staged cell
  int rows[PNROW_MAX + 1];       // crowded walk: the block's particles before each core row of fine cells
  int heavy[PP_HEAVY_LIST];      // the part's particles left to the warp walk (walk indices)
  int ncore, nring;              // staged particles of the block (slots from 0 up) and of the ring (from cap-1 down)
  int nheavy;
};
// the large brick block: staging buffers, this struct and the scans' warp sums in one SM
static_assert(PP_SMEM1B + sizeof(PPSmem) + 512 <= 227 * 1024, "the large brick block fits the shared memory of an SM");

struct PPAcc {
  unsigned long long npairs = 0, nwork = 0;
  float f2max = 0.f;
};

// Where a block stages: shared memory (levels 0-3; 16-bit slots and bin
// offsets) or a region of the global scratch (levels 4-5; 32-bit).
template <typename Idx, int kBinBits>
struct PPBuf {
  float4* pts;      // x, y, z relative to the block, particle index
  unsigned* kinfo;  // fine-cell bin | rank in the bin << kBinBits
  Idx* order;       // slots by bin, each bin's by increasing particle index
  Idx* bins;        // NF + 1 bin offsets (counts while staging)
  int cap;
};

// add n to a bin's count, return the count before: 16-bit counts two to a
// 32-bit word, or 32-bit counts
__device__ __forceinline__ unsigned bin_add(unsigned short* bins, unsigned f, unsigned n) {
  unsigned* b32 = reinterpret_cast<unsigned*>(bins);
  const unsigned sh = 16u * (f & 1u);
  return (atomicAdd(&b32[f >> 1], n << sh) >> sh) & 0xffffu;
}
__device__ __forceinline__ unsigned bin_add(unsigned* bins, unsigned f, unsigned n) { return atomicAdd(&bins[f], n); }

// Pair forces for the B[0]xB[1]xB[2] coarse cells starting at C0.  The
// particles of the block and of the fine-cell layer around it are staged
// (compacted: the block's own from slot 0 up, the ring's from cap-1 down),
// binned by fine cell with each bin in particle-index order, and every
// particle of the block then walks its 27 neighbouring fine-cell bins in
// that order.  Returns false (nothing summed) when more than cap particles
// would be staged.  Block-uniform control flow; ends with a barrier.
template <typename Idx, int kBinBits>
__device__ bool pp_block(const PPArgs& a, const int C0[3], const int B[3], PPSmem& sm,
                         const PPBuf<Idx, kBinBits>& buf, PPAcc& acc, int part = 0, int nparts = 1) {
  const Geo& g = a.g;
  const int nc = g.nc, cap = buf.cap;
  const int S0 = B[0] + 2, S1 = B[1] + 2, S2 = B[2] + 2, NS = S0 * S1 * S2;
  const int F0 = 4 * B[0] + 2, F1 = 4 * B[1] + 2, F2 = 4 * B[2] + 2, NF = F0 * F1 * F2;
  constexpr unsigned kBinMask = (1u << kBinBits) - 1u;
  float4* pts = buf.pts;
  unsigned* kinfo = buf.kinfo;
  Idx* order = buf.order;
  Idx* bins = buf.bins;
  for (int t = threadIdx.x; t < NS; t += blockDim.x) {
    int sx = t % S0, sy = (t / S0) % S1, sz = t / (S0 * S1);
    int64_t c = cell_id(g, wrap1(C0[0] + sx - 1, nc), wrap1(C0[1] + sy - 1, nc), wrap1(C0[2] + sz - 1, nc));
    sm.pref[t] = a.rhoc[c];
    sm.sstart[t] = a.cstart[c];
  }
  if constexpr (sizeof(Idx) == 2) {
    unsigned* bins32 = reinterpret_cast<unsigned*>(bins);
    for (int t = threadIdx.x; t < (NF + 2) / 2; t += blockDim.x) bins32[t] = 0u;
  } else {
    for (int t = threadIdx.x; t <= NF; t += blockDim.x) bins[t] = 0u;
  }
  if (threadIdx.x == 0) sm.ncore = sm.nring = sm.nheavy = 0;
  __syncthreads();
  const int total = block_exclusive_scan(sm.pref, NS);
  if (threadIdx.x == 0) sm.pref[NS] = total;
  __syncthreads();
  // Stage the particles whose fine cell lies in the block or its fine ring.
  // The staged cells' particles, in storage order, are split into one
  // contiguous range of whole cells per warp (about equal counts), which the
  // warp takes 32 at a time.  A fine cell's particles all come from one
  // coarse cell, so from one warp; its lanes of one pass take consecutive
  // ranks (one atomic, lane order) after those of the warp's earlier passes,
  // so every bin ends up in particle-index order whatever the block's shape,
  // level or scheduling.
  const int lane = threadIdx.x & 31, nwarp = blockDim.x >> 5, wid = threadIdx.x >> 5;
  // the first staged cell whose prefix reaches target (pref[NS] = total)
  auto first_cell = [&](int target) {
    int lo = 0, hi = NS;
    while (lo < hi) {
      const int mid = (lo + hi) >> 1;
      if (sm.pref[mid] < target) lo = mid + 1;
      else hi = mid;
    }
    return lo;
  };
  const int ca = first_cell((int)((int64_t)total * wid / nwarp));
  const int cb = wid + 1 < nwarp ? first_cell((int)((int64_t)total * (wid + 1) / nwarp)) : NS;
  const int jend = sm.pref[cb];
  const int S01 = S0 * S1;
  for (int j0 = sm.pref[ca]; j0 < jend; j0 += 32) {  // warp-uniform trip count
    const int j = j0 + lane;
    unsigned key = 0xffffffffu;  // the lane's bin, or none
    int slot = 0, pi = 0;
    float x[3] = {0.f, 0.f, 0.f};
    if (j < jend) {
      // the staged cell holding j: the last one in [ca, cb) whose prefix is <= j
      int lo = ca, hi = cb - 1;
      while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (sm.pref[mid] <= j) lo = mid;
        else hi = mid - 1;
      }
      const int t = lo;
      const int sz = t / S01, sy = (t - sz * S01) / S0, sx = t - sz * S01 - sy * S0;
      const int64_t q = sm.sstart[t] + (j - sm.pref[t]);
      const int64_t p = a.pidx ? (int64_t)__ldg(a.pidx + q) : q;
      pi = (int)p;
      const int sl[3] = {sx - 1, sy - 1, sz - 1};
      int fi[3];
      bool in = true, core = true;
#pragma unroll
      for (int d = 0; d < 3; d++) {
        x[d] = __fadd_rn((float)(4 * sl[d]), fine_off(load_code(a.xp, 3 * p + d, g.izipx), g.izipx));
        fi[d] = (int)floorf(x[d]) + 1;  // 0 .. 4B+1 inside the staged region
        in = in && fi[d] >= 0 && fi[d] <= 4 * B[d] + 1;
        core = core && fi[d] >= 1 && fi[d] <= 4 * B[d];
      }
      if (in) {
        slot = core ? atomicAdd(&sm.ncore, 1) : cap - 1 - atomicAdd(&sm.nring, 1);
        if (slot >= 0 && slot < cap) key = (unsigned)(fi[0] + F0 * (fi[1] + F1 * fi[2]));
      }
    }
    const unsigned peers = __match_any_sync(0xffffffffu, key);
    const int leader = __ffs(peers) - 1;
    unsigned base = 0;
    if (key != 0xffffffffu && lane == leader) base = bin_add(bins, key, (unsigned)__popc(peers));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (key != 0xffffffffu) {
      const unsigned r = base + (unsigned)__popc(peers & ((1u << lane) - 1u));
      pts[slot] = make_float4(x[0], x[1], x[2], __int_as_float(pi));
      kinfo[slot] = key | (r << kBinBits);
    }
  }
  __syncthreads();
  const int ncore = sm.ncore, nring = sm.nring, nst = ncore + nring;
  if (nst > cap) return false;
  if constexpr (sizeof(Idx) == 2)
    block_exclusive_scan_u16(bins, NF);
  else
    block_exclusive_scan(reinterpret_cast<int*>(bins), NF);
  if (threadIdx.x == 0) bins[NF] = (Idx)nst;
  for (int i = threadIdx.x; i < nst; i += blockDim.x) {
    const int t = i < ncore ? i : cap - nring + (i - ncore);
    const unsigned k = kinfo[t];
    order[(int)bins[k & kBinMask] + (int)(k >> kBinBits)] = (Idx)t;
  }
  // A crowded block (a quarter of a staged particle per fine cell or more:
  // a few neighbours per particle and up) walks its own particles in bin
  // order, so the lanes of a warp share their neighbour bins: the same trip
  // counts and broadcast loads.  Its particles in bin order are the core
  // rows of fine cells (4B[0] consecutive bins each) one after another.  A
  // sparse block walks its particles in slot order.  Part `part` of `nparts`
  // walks the block's particles [i0, i1) in bin order (slots differ from one
  // staging to the next; bin order does not).
  const bool crowded = 4 * nst >= NF;
  const bool by_bin = crowded || nparts > 1;
  const int RX = 4 * B[1], nrc = RX * 4 * B[2];
  if (by_bin)
    for (int r = threadIdx.x; r < nrc; r += blockDim.x) {
      const int rs = F0 * ((1 + r % RX) + F1 * (1 + r / RX));
      sm.rows[r] = (int)bins[rs + 4 * B[0] + 1] - (int)bins[rs + 1];
    }
  __syncthreads();
  if (by_bin) block_exclusive_scan(sm.rows, nrc);
  const int i0 = (int)((int64_t)ncore * part / nparts), i1 = (int)((int64_t)ncore * (part + 1) / nparts);
  // the slot of the block's i-th particle in bin order or slot order
  auto slot_of = [&](int i) -> int {
    if (!by_bin) return i;
    int lo = 0, hi = nrc;  // rows[lo] <= i < rows[hi] (rows[nrc] = ncore)
    while (hi - lo > 1) {
      const int mid = (lo + hi) >> 1;
      if (sm.rows[mid] <= i) lo = mid;
      else hi = mid;
    }
    const int rs = F0 * ((1 + lo % RX) + F1 * (1 + lo / RX));
    return (int)order[(int)bins[rs + 1] + (i - sm.rows[lo])];
  };
  // the bin offset of neighbour row r (dz-major): its bins dx = -1..1 are
  // consecutive, one range [bins[f + off - 1], bins[f + off + 2])
  auto row_off = [&](int r) { return F0 * ((r % 3 - 1) + F1 * (r / 3 - 1)); };
  // thread walks: one particle per thread (in a crowded block, the light ones)
  for (int i = i0 + (int)threadIdx.x; i < i1; i += blockDim.x) {
    const int t = slot_of(i);
    const float4 q = pts[t];
    const int f = (int)(kinfo[t] & kBinMask);
    long long Q[3] = {0, 0, 0};
    float s[3] = {0.f, 0.f, 0.f}, c[3] = {0.f, 0.f, 0.f};
    int cnt = 0;
    if (crowded) {
      int E = 0;
      for (int r = 0; r < 9; r++) E += (int)bins[f + row_off(r) + 2] - (int)bins[f + row_off(r) - 1];
      if (E >= a.heavy) {  // left to the warp walk below
        const int h = atomicAdd(&sm.nheavy, 1);
        if (h < PP_HEAVY_LIST) sm.heavy[h] = i;
        continue;
      }
      acc.npairs += (unsigned)E;
      for (int r = 0; r < 9; r++) {
        const int k1 = (int)bins[f + row_off(r) + 2];
        for (int k = (int)bins[f + row_off(r) - 1]; k < k1; k++) {
          const float4 o = pts[order[k]];
          pair_force(a, o.x - q.x, o.y - q.y, o.z - q.z, s, c);
          if (++cnt == PP_CHUNK) {
            pp_fold(Q, s, c);
            cnt = 0;
          }
        }
      }
    } else {
      // the nine ranges as one loop over their concatenation: a warp runs as
      // many passes as its busiest lane has pairs, not the sum over rows of
      // each row's busiest lane
      int rk = 0, k = 0, kend = 0;
      for (;;) {
        while (k == kend && rk < 9) {
          k = (int)bins[f + row_off(rk) - 1];
          kend = (int)bins[f + row_off(rk) + 2];
          acc.npairs += (unsigned)(kend - k);
          rk++;
        }
        if (k == kend) break;
        const float4 o = pts[order[k++]];
        pair_force(a, o.x - q.x, o.y - q.y, o.z - q.z, s, c);
        if (++cnt == PP_CHUNK) {
          pp_fold(Q, s, c);
          cnt = 0;
        }
      }
    }
    if (cnt) pp_fold(Q, s, c);
    acc.nwork++;
    acc.f2max = fmaxf(acc.f2max, pp_store_force(a, (int64_t)__float_as_int(q.w), Q));
  }
  // warp walks: a crowded block's heavy particles (a.heavy entries or more),
  // one per warp, lane l taking chunks l, l+32, ...; the chunks' fixed-point
  // values are summed across the warp, so the result is the thread walk's to
  // the bit
  __syncthreads();
  const int nheavy = sm.nheavy;
  if (crowded && nheavy > 0) {
    // the listed heavy particles, or (list overflowed) every particle of the part
    const bool listed = nheavy <= PP_HEAVY_LIST;
    const int lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    for (int h = (int)(threadIdx.x >> 5); h < (listed ? nheavy : i1 - i0); h += nw) {
      const int i = listed ? sm.heavy[h] : i0 + h;
      const int t = slot_of(i);
      const int f = (int)(kinfo[t] & kBinMask);
      int E = 0;
      for (int r = 0; r < 9; r++) E += (int)bins[f + row_off(r) + 2] - (int)bins[f + row_off(r) - 1];
      if (E < a.heavy) continue;  // warp-uniform: every lane has the same E
      const float4 q = pts[t];
      const int J = (E + PP_CHUNK - 1) / PP_CHUNK;
      long long Q[3] = {0, 0, 0};
      for (int j0 = 0; j0 < J; j0 += 32) {
        const int j = j0 + lane;
        float s[3] = {0.f, 0.f, 0.f}, c[3] = {0.f, 0.f, 0.f};
        if (j < J) {
          // entry j*PP_CHUNK of the concatenated rows, then PP_CHUNK entries on
          int e = j * PP_CHUNK, r = 0, k = 0, kend = 0;
          for (;;) {
            k = (int)bins[f + row_off(r) - 1];
            kend = (int)bins[f + row_off(r) + 2];
            if (e < kend - k) break;
            e -= kend - k;
            r++;
          }
          k += e;
          for (int m = 0; m < PP_CHUNK; m++) {
            while (k == kend && r < 8) {
              r++;
              k = (int)bins[f + row_off(r) - 1];
              kend = (int)bins[f + row_off(r) + 2];
            }
            if (k == kend) break;
            const float4 o = pts[order[k++]];
            pair_force(a, o.x - q.x, o.y - q.y, o.z - q.z, s, c);
          }
        }
#pragma unroll
        for (int d = 0; d < 3; d++) {
          long long v = j < J ? to_fix(__fsub_rn(s[d], c[d])) : 0;
          for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
          Q[d] += v;
        }
      }
      if (lane == 0) {
        acc.npairs += (unsigned)E;
        acc.nwork++;
        acc.f2max = fmaxf(acc.f2max, pp_store_force(a, (int64_t)__float_as_int(q.w), Q));
      }
    }
  }
  __syncthreads();
  return true;
}

// The next item of a listed level for this block: the lists are shared out
// as blocks finish (a dense item can take many times another's time).
__device__ __forceinline__ int pp_next(int* counter, int* s_it) {
  if (threadIdx.x == 0) *s_it = atomicAdd(counter, 1);
  __syncthreads();
  const int it = *s_it;
  __syncthreads();
  return it;
}

// The next (item, part) of a listed level whose items are split into parts
// (each part walks a slice of the item's particles, on its own SM): a cursor
// runs over the n items, each item's word counts its parts (low 8 bits) and
// the parts claimed so far (above).  Lock-free: each pass either claims a
// part or moves the cursor past an item whose parts are all claimed.
__device__ __forceinline__ bool pp_next_part(int* cursor, int n, int* word, int* s3, int& it, int& part,
                                             int& nparts) {
  if (threadIdx.x == 0) {
    int ri = -1, rp = 0, rn = 1;
    for (;;) {
      const int cur = *(volatile int*)cursor;
      if (cur >= n) break;
      const int w = atomicAdd(&word[cur], 256);
      if ((w >> 8) < (w & 255)) {
        ri = cur;
        rp = w >> 8;
        rn = w & 255;
        break;
      }
      atomicCAS(cursor, cur, cur + 1);
    }
    s3[0] = ri;
    s3[1] = rp;
    s3[2] = rn;
  }
  __syncthreads();
  it = s3[0];
  part = s3[1];
  nparts = s3[2];
  __syncthreads();
  return it >= 0;
}

// List an item that did not fit (thread 0 of its block) for level l+1, with
// the number of parts that level splits it into: about 2^22 staged-pair
// candidates (core x staged particles) a part, 32 core particles at least.
__device__ __forceinline__ void pp_list_item(const PPArgs& a, int l, int item, int ncore, int nst, bool split) {
  const int idx = atomicAdd(&a.nlist[l], 1);
  a.list[l][idx] = item;
  int64_t P = 1;
  if (split) {
    P = (((int64_t)ncore * nst) >> 22) + 1;
    P = min(P, (int64_t)max(1, ncore / 32));
    P = max((int64_t)1, min(P, (int64_t)a.max_parts));
  }
  a.lpart[l][idx] = (int)P;
}

// Levels 0-3 (shared-memory staging).  Level 0: a brick per block; level 2:
// the cells of the bricks level 1 could not hold; levels 1 and 3: listed
// bricks / cells in parts.  What does not fit is listed for the next level.
template <int kLevel, int CAP, int NT>
__global__ void __launch_bounds__(NT, NT <= 128 ? 8 : (NT <= 256 ? 4 : 1)) k_pp_level(PPArgs a) {
  __shared__ PPSmem sm;
  __shared__ int s3[3];
  extern __shared__ float4 dyn[];
  const Geo& g = a.g;
  const int nc = g.nc, nb = a.nb;
  PPBuf<unsigned short, 13> buf;
  buf.pts = dyn;
  buf.kinfo = reinterpret_cast<unsigned*>(dyn + CAP);
  buf.order = reinterpret_cast<unsigned short*>(buf.kinfo + CAP);
  buf.bins = buf.order + CAP;
  buf.cap = CAP;
  PPAcc acc;
  auto brick = [&](int b, int C0[3], int B[3]) {
    C0[0] = (b % nb) * PB;
    C0[1] = ((b / nb) % nb) * PB;
    C0[2] = (b / (nb * nb)) * PB;
    for (int d = 0; d < 3; d++) B[d] = min(PB, nc - C0[d]);
  };
  if (kLevel == 0 || kLevel == 2) {
    const int n = kLevel == 0 ? nb * nb * nb : a.nlist[1] * PNCORE_MAX;
    for (int it = kLevel == 0 ? (int)blockIdx.x : pp_next(a.nlist + 5 + kLevel, &s3[0]); it < n;
         it = kLevel == 0 ? it + (int)gridDim.x : pp_next(a.nlist + 5 + kLevel, &s3[0])) {
      int C0[3], B[3];
      int item;  // what is listed for the next level if this one does not fit
      if (kLevel == 0) {
        brick(it, C0, B);
        item = it;
      } else {
        const int b = a.list[1][it / PNCORE_MAX], l = it % PNCORE_MAX;
        C0[0] = (b % nb) * PB + l % PB;
        C0[1] = ((b / nb) % nb) * PB + (l / PB) % PB;
        C0[2] = (b / (nb * nb)) * PB + l / (PB * PB);
        if (C0[0] >= nc || C0[1] >= nc || C0[2] >= nc) continue;
        item = (int)cell_id(g, C0[0], C0[1], C0[2]);
        B[0] = B[1] = B[2] = 1;
      }
      if (!pp_block(a, C0, B, sm, buf, acc)) {
        if (threadIdx.x == 0) pp_list_item(a, kLevel, item, sm.ncore, sm.ncore + sm.nring, true);
        __syncthreads();
      }
    }
  } else {
    const int n = a.nlist[kLevel - 1];
    int it, part, np;
    while (pp_next_part(a.nlist + 5 + kLevel, n, a.lpart[kLevel - 1], s3, it, part, np)) {
      const int item = a.list[kLevel - 1][it];
      int C0[3], B[3];
      if (kLevel == 1) {
        brick(item, C0, B);
      } else {
        cell_coords(g, item, C0[0], C0[1], C0[2]);
        B[0] = B[1] = B[2] = 1;
      }
      if (!pp_block(a, C0, B, sm, buf, acc, part, np)) {
        // level 2 takes a brick cell by cell (no parts), level 4 a cell in parts
        if (threadIdx.x == 0 && part == 0) pp_list_item(a, kLevel, item, sm.ncore, sm.ncore + sm.nring, kLevel == 3);
        __syncthreads();
      }
    }
  }
  pp_reduce(a, acc.npairs, acc.nwork, acc.f2max);
}

// Levels 4 and 5: listed cells staged in the global scratch (32-bit slots
// and offsets; the bins stay in shared memory).  Level 4 gives each block an
// equal region and takes its cells in parts; a cell that does not fit goes
// to level 5, one block with the whole scratch; a cell even that cannot
// hold is counted as an overflow and its particles keep no PP force (the
// call reports it).
template <int kLevel>
__global__ void __launch_bounds__(PP_THREADS1) k_pp_global(PPArgs a) {
  __shared__ PPSmem sm;
  __shared__ unsigned bins[PNF1 + 2];
  __shared__ int s3[3];
  const Geo& g = a.g;
  const int n = a.nlist[kLevel - 1];
  const int64_t share = kLevel == 4 ? a.scr_cap / gridDim.x : a.scr_cap;
  const int64_t off = kLevel == 4 ? share * blockIdx.x : 0;
  PPBuf<unsigned, 8> buf;
  buf.pts = a.scr_pts + off;
  buf.kinfo = a.scr_kinfo + off;
  buf.order = a.scr_order + off;
  buf.bins = bins;
  buf.cap = (int)share;
  PPAcc acc;
  int it, part, np;
  while (pp_next_part(a.nlist + 5 + kLevel, n, a.lpart[kLevel - 1], s3, it, part, np)) {
    const int item = a.list[kLevel - 1][it];
    int C0[3];
    const int B[3] = {1, 1, 1};
    cell_coords(g, item, C0[0], C0[1], C0[2]);
    if (!pp_block(a, C0, B, sm, buf, acc, part, np)) {
      if (threadIdx.x == 0 && part == 0) {
        if (kLevel == 4) pp_list_item(a, 4, item, sm.ncore, sm.ncore + sm.nring, false);
        else atomicAdd(&a.st->pp_overflow, 1u);
      }
      __syncthreads();
    }
  }
  pp_reduce(a, acc.npairs, acc.nwork, acc.f2max);
}

// forced start level (tests): list every brick, or every cell, in `parts` parts
__global__ void k_pp_list_all(int* list, int* word, int n, int* count, int parts) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    list[i] = i;
    word[i] = parts;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) *count = n;
}

// ------------------------------------------------------------- prefilter
// A particle's list holds the particles of its 27 neighbouring fine cells
// (ext_pp_force.f90:94-96); when that is the particle itself alone, its pair
// force is zero and its list has one entry.  The relation is symmetric, so
// every neighbour of a particle with a longer list has one too: staging only
// the particles with a neighbour ("active") gives each of them the same list
// in the same order as staging every particle, hence the same bits.  Per
// coarse cell a 64-bit mask holds the occupied fine sub-cells (bit x + 4y +
// 16z) and a second those held by two particles or more; each particle then
// tests the sub-cells within one fine cell of its own, in its cell and the
// (up to 7) neighbouring cells they reach.  The active particles are
// compacted in storage order with per-cell counts and starts, which the
// staging kernels read in place of rhoc and cstart.
struct PPFilter {
  Geo g;
  int64_t np, ncells;
  const void* xp;
  const int32_t* pcell;
  const int32_t* rhoc;
  const int64_t* cstart;
  unsigned long long* occ;    // ncells occupied masks, then ncells multiple masks
  unsigned* act;              // a bit per particle
  int32_t* wcnt;              // active particles per word of act
  const int64_t* wstart;      // exclusive scan of wcnt
  int32_t* arhoc;
  int64_t* acstart;
  int32_t* aidx;
  DevStats* st;
};

// fine sub-cell of particle p in its coarse cell: the top two bits of each
// unsigned position code (floor(4*(code+0.5)/2^(8*izipx)), pm.f90 / ext_pp_force.f90:91)
__device__ __forceinline__ void sub_cell(const void* xp, int64_t p, int izipx, int s[3]) {
  const int m = (1 << (8 * izipx)) - 1, sh = 8 * izipx - 2;
#pragma unroll
  for (int d = 0; d < 3; d++) s[d] = (load_code(xp, 3 * p + d, izipx) & m) >> sh;
}

// a cell's occupied sub-cells and those held twice or more: one thread per
// coarse cell over its particles (no atomics; every cell's words written)
__global__ void __launch_bounds__(256) k_pp_occ(PPFilter f) {
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < f.ncells; c += (int64_t)gridDim.x * blockDim.x) {
    const int n = __ldg(f.rhoc + c);
    const int64_t p0 = __ldg(f.cstart + c);
    unsigned long long m = 0ull, t = 0ull;
    for (int j = 0; j < n; j++) {
      int s[3];
      sub_cell(f.xp, p0 + j, f.g.izipx, s);
      const unsigned long long b = 1ull << (s[0] + 4 * (s[1] + 4 * s[2]));
      t |= m & b;
      m |= b;
    }
    f.occ[c] = m;
    f.occ[f.ncells + c] = t;
  }
}

// the part of cell_id that coordinate d contributes (cell_id is their sum:
// ix + nt*iy + nt^2*iz + nt^3*(tx + nnt*ty + nnt^2*tz))
__device__ __forceinline__ uint32_t cell_part(const Geo& g, int d, int gc) {
  const uint32_t t = fdiv((uint32_t)gc, g.dnt), i = (uint32_t)gc - t * (uint32_t)g.nt;
  const uint32_t nt = (uint32_t)g.nt, nt3 = nt * nt * nt, nnt = (uint32_t)g.nnt;
  if (d == 0) return i + nt3 * t;
  if (d == 1) return nt * i + nt3 * nnt * t;
  return nt * nt * i + nt3 * nnt * nnt * t;
}

// Sub-cell bit operations (bit x + 4y + 16z): the layer x = 0 (y = 0, z = 0)
// of a cell, and moves of every bit by one sub-cell along a dimension
// (bits leaving the cell drop).
__host__ __device__ constexpr unsigned long long lay0(int d) {
  return d == 0 ? 0x1111111111111111ull : (d == 1 ? 0x000F000F000F000Full : 0x000000000000FFFFull);
}
__host__ __device__ constexpr int sub_stride(int d) { return d == 0 ? 1 : (d == 1 ? 4 : 16); }
__device__ __forceinline__ unsigned long long sub_up(unsigned long long m, int d) {   // to coordinate + 1
  return (m << sub_stride(d)) & ~lay0(d);
}
__device__ __forceinline__ unsigned long long sub_down(unsigned long long m, int d) {  // to coordinate - 1
  return (m >> sub_stride(d)) & ~(lay0(d) << (3 * sub_stride(d)));
}
__device__ __forceinline__ unsigned long long sub_ex(unsigned long long m, int d) { return sub_up(m, d) | sub_down(m, d); }
__device__ __forceinline__ unsigned long long sub_dil(unsigned long long m, int d) { return m | sub_ex(m, d); }

// Per coarse cell, the sub-cells whose 26 neighbouring fine cells (its own
// and the 26 surrounding coarse cells') hold a particle, or that hold two
// themselves: a particle there has a neighbour besides itself.  Within the
// cell, a neighbour differs by one in z (any x, y), or in y only (any x), or
// in x only; a surrounding cell contributes its facing layer(s), moved to
// the adjoining layer(s) of this cell and spread by one in the other
// dimensions.  Written over the cell's multiple mask, which no other cell
// reads.
__global__ void __launch_bounds__(256) k_pp_nbmask(PPFilter f) {
  const Geo& g = f.g;
  const int nc = g.nc;
  unsigned long long nact = 0, nidle = 0;
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < f.ncells; c += (int64_t)gridDim.x * blockDim.x) {
    int gc[3];
    cell_coords(g, c, gc[0], gc[1], gc[2]);
    uint32_t part[3][3];  // coordinate - 1, itself, + 1
#pragma unroll
    for (int d = 0; d < 3; d++)
      for (int o = -1; o <= 1; o++) part[d][o + 1] = cell_part(g, d, wrap1(gc[d] + o, nc));
    const unsigned long long own = __ldg(f.occ + c);
    const unsigned long long dxo = sub_dil(own, 0);
    unsigned long long e = sub_ex(sub_dil(dxo, 1), 2) | sub_ex(dxo, 1) | sub_ex(own, 0);
#pragma unroll
    for (int k = 0; k < 27; k++) {
      const int o[3] = {k % 3 - 1, (k / 3) % 3 - 1, k / 9 - 1};
      if (o[0] == 0 && o[1] == 0 && o[2] == 0) continue;
      unsigned long long l = __ldg(f.occ + (part[0][o[0] + 1] + part[1][o[1] + 1] + part[2][o[2] + 1]));
#pragma unroll
      for (int d = 0; d < 3; d++) {
        if (o[d] < 0) l = (l >> (3 * sub_stride(d))) & lay0(d);                              // its layer 3 to our layer 0
        else if (o[d] > 0) l = (l << (3 * sub_stride(d))) & (lay0(d) << (3 * sub_stride(d)));  // its layer 0 to our layer 3
      }
#pragma unroll
      for (int d = 0; d < 3; d++)
        if (o[d] == 0) l = sub_dil(l, d);
      e |= l;
    }
    // then the cell's own particles: active where their sub-cell's bit is
    // set (act and wcnt zeroed before the launch)
    const unsigned long long a = e | __ldg(f.occ + f.ncells + c);
    const int n = __ldg(f.rhoc + c);
    const int64_t p0 = __ldg(f.cstart + c);
    for (int j = 0; j < n; j++) {
      const int64_t p = p0 + j;
      int s[3];
      sub_cell(f.xp, p, g.izipx, s);
      if ((a >> (s[0] + 4 * (s[1] + 4 * s[2]))) & 1ull) {
        atomicOr(&f.act[p >> 5], 1u << (p & 31));
        atomicAdd(&f.wcnt[p >> 5], 1);
        nact++;
      } else {
        nidle++;
      }
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    nact += __shfl_xor_sync(0xffffffffu, nact, o);
    nidle += __shfl_xor_sync(0xffffffffu, nidle, o);
  }
  if ((threadIdx.x & 31) == 0) {
    // a particle left out has the one entry of itself and a zero force (itest1 counts it)
    if (nidle) {
      atomicAdd(&f.st->npairs, nidle);
      atomicAdd(&f.st->itest1, nidle);
    }
    if (nact) atomicAdd(&f.st->pp_active, nact);
  }
}

// active particles before storage position q
__device__ __forceinline__ int64_t act_prefix(const PPFilter& f, int64_t q) {
  const int64_t w = q >> 5;
  const int r = (int)(q & 31);
  return r == 0 ? __ldg(f.wstart + w) : __ldg(f.wstart + w) + __popc(__ldg(f.act + w) & ((1u << r) - 1u));
}

__global__ void __launch_bounds__(256) k_pp_acells(PPFilter f) {
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < f.ncells; c += (int64_t)gridDim.x * blockDim.x) {
    const int64_t s0 = __ldg(f.cstart + c);
    const int64_t a0 = act_prefix(f, s0);
    f.acstart[c] = a0;
    f.arhoc[c] = (int32_t)(act_prefix(f, s0 + __ldg(f.rhoc + c)) - a0);
  }
}

__global__ void __launch_bounds__(256) k_pp_aidx(PPFilter f) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < f.np; p += (int64_t)gridDim.x * blockDim.x) {
    const unsigned w = __ldg(f.act + (p >> 5));
    const int r = (int)(p & 31);
    if ((w >> r) & 1u) f.aidx[__ldg(f.wstart + (p >> 5)) + __popc(w & ((1u << r) - 1u))] = (int32_t)p;
  }
}

}  // namespace

// whether this PP launch runs the prefilter: automatic while under half of
// the particles had a neighbour at the last filtered call (a uniform early
// state has about one in ten), re-tried every 16th call otherwise; always
// inside a captured graph, where no count comes back to the host
static bool pp_filter_on(cube_ctx* c) {
  if (!c->pp_occ || c->p.nc < 4 || c->opt_pp_filter == 1) return false;
  if (c->graph_mode) return true;
  if (c->opt_pp_filter == 2 || c->pp_active_frac < 0.5f) return true;
  return ++c->pp_unfiltered % 16 == 0;
}

// every PP launch on c->stream (stats in c->dstats); the host reads nothing
int cube_pp_launch(cube_ctx* c, float a_mid, float dt, bool defer_kick) {
  if (!c->fpp) return cube_fail(c, CUBE_ERR_ARG, "PP is off for this context (pp_on = 0)");
  PPArgs a{};
  int r;
  if (c->graph_mode) {
    cube_codec_view_dev(c, 0, &c->sd->h.cf_vi, &a.cv);
    a.sd = c->sd;
  } else {
    r = cube_codec_pair(c, c->sigma_vi, c->sigma_vi, &a.cv, nullptr);
    if (r) return r;
  }
  CUBE_CUDA(c, cudaMemsetAsync(c->dstats, 0, sizeof(DevStats), c->stream));
  a.g = make_geo(c);
  a.np = c->np;
  a.xp = c->xp[c->cur];
  a.vp = c->vp[c->cur];
  a.rhoc = c->rhoc[c->cur];
  a.cstart = c->cstart[c->cur];
  a.mass = c->p.mass_p;
  a.rsoft = c->p.rsoft;
  a.inv_cut = 1.0f / (float)c->p.nf_cutoff;
  a.kick = (((double)a_mid * (double)dt) / 6.0) / (double)CUBE_PI_F;
  a.kick_f = (float)a.kick;
  a.exact_only = c->opt_exact_kicks;
  a.fpp = c->fpp;
  a.st = c->dstats;
  a.nb = (c->p.nc + PB - 1) / PB;
  int64_t nbrick = (int64_t)a.nb * a.nb * a.nb;
  if (nbrick > c->pp_brick_cap) return cube_fail(c, CUBE_ERR_ARG, "PP brick list too small");
  for (int l = 0; l < 5; l++) {
    a.list[l] = c->pp_list[l];
    a.lpart[l] = c->pp_lpart[l];
  }
  a.heavy = c->opt_pp_heavy > 0 ? c->opt_pp_heavy : PP_HEAVY;
  a.max_parts = c->opt_pp_parts > 0 ? c->opt_pp_parts : 255;
  a.nlist = c->pp_nlist;
  a.scr_cap = c->pp_scr_cap;
  a.scr_pts = c->pp_scr_pts;
  a.scr_kinfo = reinterpret_cast<unsigned*>(c->pp_scr_pts + c->pp_scr_cap);
  a.scr_order = a.scr_kinfo + c->pp_scr_cap;
  CUBE_CUDA(c, cudaMemsetAsync(c->pp_nlist, 0, 11 * sizeof(int), c->stream));
  a.pidx = nullptr;
  a.act = nullptr;
  a.nact = nullptr;
  c->pp_act_valid = pp_filter_on(c) && a.cv.rt;
  auto k0 = k_pp_level<0, PP_CAP, PP_THREADS>;
  auto k1 = k_pp_level<1, PP_CAP1, PP_THREADS1>;
  auto k2 = k_pp_level<2, PP_CAP, PP_THREADS>;
  auto k3 = k_pp_level<3, PP_CAP1, PP_THREADS1>;
  const int persist = cube_grid((int64_t)1 << 40, 1, 4), one_per_sm = cube_grid((int64_t)1 << 40, 1, 1);
  cube_phase_begin(c, PH_PP);
  if (c->pp_act_valid) {
    PPFilter f;
    f.g = a.g;
    f.np = c->np;
    f.ncells = c->ncells;
    f.xp = a.xp;
    f.pcell = c->pcell[c->cur];
    f.rhoc = a.rhoc;
    f.cstart = a.cstart;
    f.occ = c->pp_occ;
    f.act = c->pp_act;
    f.wcnt = c->pp_wcnt;
    f.wstart = c->pp_wstart;
    f.arhoc = c->pp_arhoc;
    f.acstart = c->pp_acstart;
    f.aidx = c->pp_aidx;
    f.st = c->dstats;
    const int64_t nw = (c->np + 31) / 32;
    k_pp_occ<<<cube_grid(c->ncells, 256), 256, 0, c->stream>>>(f);
    CUBE_CUDA(c, cudaMemsetAsync(c->pp_act, 0, 4 * (size_t)nw, c->stream));
    CUBE_CUDA(c, cudaMemsetAsync(c->pp_wcnt, 0, 4 * (size_t)nw, c->stream));
    k_pp_nbmask<<<cube_grid(c->ncells, 256), 256, 0, c->stream>>>(f);
    if (c->np > 0) {
      r = cube_scan_counts(c, c->pp_wcnt, c->pp_wstart, nw);
      if (r) return r;
      k_pp_aidx<<<cube_grid(c->np, 256), 256, 0, c->stream>>>(f);
    } else {
      CUBE_CUDA(c, cudaMemsetAsync(c->pp_wstart, 0, 8, c->stream));
    }
    k_pp_acells<<<cube_grid(c->ncells, 256), 256, 0, c->stream>>>(f);
    a.rhoc = c->pp_arhoc;
    a.cstart = c->pp_acstart;
    a.pidx = c->pp_aidx;
    a.act = c->pp_act;
    a.nact = c->pp_wstart + nw;
  }
  // a forced first level lists everything for it (tests of the dense paths)
  const int start = c->opt_pp_level;
  if (start == 1 || start == 2)
    k_pp_list_all<<<cube_grid(nbrick, 256), 256, 0, c->stream>>>(c->pp_list[start - 1], c->pp_lpart[start - 1],
                                                                 (int)nbrick, c->pp_nlist + start - 1,
                                                                 start == 1 ? 3 : 1);
  else if (start >= 3)  // cells
    k_pp_list_all<<<cube_grid(c->ncells, 256), 256, 0, c->stream>>>(c->pp_list[start - 1], c->pp_lpart[start - 1],
                                                                     (int)c->ncells, c->pp_nlist + start - 1,
                                                                     start == 5 ? 1 : 3);
  if (start <= 0) {
    if (c->pp_act_valid && !c->graph_mode && c->pp_active_frac < PP_SPARSE_FRAC)
      k_pp_level<0, PP_CAP_S, PP_THREADS_S><<<(unsigned)nbrick, PP_THREADS_S, PP_SMEM_S, c->stream>>>(a);
    else
      k0<<<(unsigned)nbrick, PP_THREADS, PP_SMEM, c->stream>>>(a);
  }
  if (start <= 1) k1<<<one_per_sm, PP_THREADS1, PP_SMEM1B, c->stream>>>(a);
  if (start <= 2) k2<<<persist, PP_THREADS, PP_SMEM, c->stream>>>(a);
  if (start <= 3) k3<<<one_per_sm, PP_THREADS1, PP_SMEM1, c->stream>>>(a);
  // level 4: a block per SM, each region at least twice level 3's room
  const int g4 = (int)std::max<int64_t>(1, std::min<int64_t>(one_per_sm, c->pp_scr_cap / (2 * PP_CAP1)));
  if (start <= 4) k_pp_global<4><<<g4, PP_THREADS1, 0, c->stream>>>(a);
  k_pp_global<5><<<1, PP_THREADS1, 0, c->stream>>>(a);
  if (c->pp_act_valid) {
    // the active particles' kick now (a deferred fine kick then gives the
    // others their zero-kick codes); the others' here when not deferred
    k_pp_kick_active<<<cube_grid(c->np, 256), 256, 0, c->stream>>>(a);
    if (!defer_kick) k_pp_kick_idle<<<cube_grid(c->np, 256), 256, 0, c->stream>>>(a);
  } else if (!defer_kick) {
    k_pp_kick<<<cube_grid(c->np, 256), 256, 0, c->stream>>>(a);
  }
  CUBE_CUDA(c, cudaGetLastError());
  cube_phase_end(c, PH_PP);
  if (c->graph_mode) {
    CUBE_CUDA(c, cudaMemcpyAsync(&c->sout->pp, c->dstats, sizeof(DevStats), cudaMemcpyDeviceToDevice, c->stream));
    return CUBE_OK;
  }
  CUBE_CUDA(c, cudaMemcpyAsync(c->pp_nlist_host, c->pp_nlist, 5 * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  return CUBE_OK;
}

// the staging kernels' shared-memory sizes, set once per context (the
// device's function attributes outlive the call)
int cube_pp_init(cube_ctx* c) {
  CUBE_CUDA(c, cudaFuncSetAttribute(k_pp_level<0, PP_CAP, PP_THREADS>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)PP_SMEM));
  CUBE_CUDA(c, cudaFuncSetAttribute(k_pp_level<1, PP_CAP1, PP_THREADS1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)PP_SMEM1B));
  CUBE_CUDA(c, cudaFuncSetAttribute(k_pp_level<2, PP_CAP, PP_THREADS>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)PP_SMEM));
  CUBE_CUDA(c, cudaFuncSetAttribute(k_pp_level<3, PP_CAP1, PP_THREADS1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)PP_SMEM1));
  return CUBE_OK;
}

// the stats of the launches above, once they are done (itest1 check of
// ext_pp_force.f90:141)
int cube_pp_finish(cube_ctx* c, cube_stats* st) {
  int r = cube_stats_fetch(c);
  if (r) return r;
  if (c->hstats->pp_overflow)
    return cube_fail(c, CUBE_ERR_PP_OVERFLOW, "PP: " + std::to_string(c->hstats->pp_overflow) +
                                                   " cell(s) with their fine-cell ring hold more particles than the " +
                                                   std::to_string(c->pp_scr_cap) + " the PP scratch stages");
  if ((int64_t)c->hstats->itest1 != c->np)
    return cube_fail(c, CUBE_ERR_COUNT_MISMATCH, "PP updated a different number of particles than nplocal");
  if (c->pp_act_valid && c->np > 0) {
    c->pp_active_frac = (float)((double)c->hstats->pp_active / (double)c->np);
    if (c->pp_active_frac < 0.5f) c->pp_unfiltered = 0;
  }
  if (st) {
    st->f2_max_pp = bits_float(c->hstats->f2_pp_bits);
    st->npairs = (int64_t)c->hstats->npairs;
    st->itest1 = (int64_t)c->hstats->itest1;
    st->pp_dense_bricks = c->pp_nlist_host[0];
  }
  return CUBE_OK;
}

int cube_pp_impl(cube_ctx* c, float a_mid, float dt, cube_stats* st) {
  int r = cube_pp_launch(c, a_mid, dt);
  if (r || c->graph_mode) return r;
  return cube_pp_finish(c, st);
}
