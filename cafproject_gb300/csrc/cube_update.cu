// cube_update.cu -- update_xp (update_particle.f90:16-256) as a GB300
// counting re-sort that reproduces the reference's integer state bit for bit.
//
// The reference visits, per tile, every particle of the tile's extended
// region (local cells 1-ncb..nt+ncb) in the layered order
//   ilayer, k (stride nlayer), j, i, l          (update_particle.f90:55-61)
// computes its destination ig=ceiling(xq+deltax) in that tile's frame, and
// keeps it when ig is a physical cell.  The rank of a particle inside its
// destination cell -- and the order in which vfield_new sums its velocity --
// is that visit order.  Here:
//   U1 (per particle)   destination cell(s) in every frame that sees it,
//                       exactly as the reference rounds in that frame;
//   U2 (per cell)       walk the (2R+1)^3 source cells in the destination
//                       frame's visit order, assign ranks, accumulate vfield;
//   scan                new spine (cell starts);
//   U3 (per particle)   write the re-encoded particle at start+rank.
#include <cmath>
#include <vector>

#include "cube_internal.cuh"

namespace {

constexpr double kWeightV = (double)0.1f;  // real(8),parameter :: weight_v=0.1 (a real(4) literal)

struct UpdArgs {
  Geo g;
  int64_t np, ncells;
  float dt_mid;
  int nlayer;
  const void* xp;
  const void* vp;
  const int32_t* pid;
  const int32_t* pcell;
  const float* vfield;
  const int64_t* cstart;
  CodecView cv;       // decode / encode tables for sigma_vi
  int exact_only;     // skip every certified fast path (FP64 expressions only)
  int32_t* dest;
  uint8_t* dframe;
  uint8_t* doff;
  uint16_t* lrank;
  uint16_t* offc;    // [o * ncells + S]: per neighbour o, one plane over the source cells
  int32_t* perm;
  uint32_t* rank;
  int4* xtra;
  int64_t xtra_cap;
  DevStats* st;
  // outputs
  int32_t* cnt_new;
  float* vfield_new;
  const int64_t* cstart_new;
  void* xp_new;
  void* vp_new;
  int32_t* pid_new;
  int32_t* pcell_new;
  const StepDev* sd;  // graph mode: dt_mid and nlayer from the device
  int32_t* vdense;    // destination cells over VF_DENSE particles, for k_vfield_dense
  int64_t p_lo;       // k_dest: first particle of this launch (particles [p_lo, np))
};

__device__ __forceinline__ float dtm(const UpdArgs& a) { return a.sd ? __ldg(&a.sd->h.dt_mid) : a.dt_mid; }
__device__ __forceinline__ int nlay(const UpdArgs& a) { return a.sd ? __ldg(&a.sd->h.nlayer) : a.nlayer; }
// graph mode runs both rank paths' launches; each skips itself on the device:
// the walker unless the counting path flagged itself inapplicable, the
// counting path's placement when it did
__device__ __forceinline__ bool counting_failed(const UpdArgs& a) { return (*(volatile int*)&a.st->flags & 12) != 0; }


// global coarse coordinate of tile-local cell l (1-based) of tile coordinate t
__device__ __forceinline__ int glob(const Geo& g, int t, int l) { return wrap1(t * g.nt + l - 1, g.nc); }

// frame offset code (0,1,2 for -nt,0,+nt) at which a tile sees global cell s
// at tile-local coordinate l
__device__ __forceinline__ int frame_code(const Geo& g, int l, int s) {
  int T, Ls;
  tile_local(g, s, T, Ls);
  int o = l - Ls;
  return o == 0 ? 1 : (o > 0 ? 2 : 0);
}

// The reference's FP64 expressions, taken only by lanes whose fast path could
// not be certified.  They are separate non-inlined functions so the compiler
// cannot hoist their double conversions into the common path (GB300 runs
// float<->double conversions on its narrow double-precision pipe).

// ig=ceiling(xq+deltax) (update_particle.f90:66-70)
__device__ __noinline__ int dest_exact(CodecView cv, int vcode, float vfd, float dt_mid, int Ls, float offf) {
  double v = __dadd_rn(codec_decode(cv, vcode), (double)vfd);
  double deltax = __dmul_rn(__dmul_rn((double)dt_mid, v), 0.25);
  double xq = __dadd_rn((double)(Ls - 1), (double)offf);
  return (int)ceil(__dadd_rn(xq, deltax));
}
// vfield_new=vfield_new+vreal rounded to real(4) (update_particle.f90:72)
__device__ __noinline__ float accumulate_exact(CodecView cv, int vcode, float vfs, float acc) {
  double v = __dadd_rn(codec_decode(cv, vcode), (double)vfs);
  return __double2float_rn(__dadd_rn((double)acc, v));
}
// vfield_new/(rhoce+weight_v) rounded to real(4) (update_particle.f90:81-83)
__device__ __noinline__ float quotient_exact(float acc, uint32_t cnt) {
  return __double2float_rn(__ddiv_rn((double)acc, __dadd_rn((double)cnt, kWeightV)));
}
// U1: destination of every particle in every frame that sees it.
__global__ void k_dest(UpdArgs a) {
  const Geo& g = a.g;
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  int local_max = 0;
  for (int64_t p = a.p_lo + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < a.np; p += stride) {
    int64_t cell = a.pcell[p];
    int gc[3];
    cell_coords(g, cell, gc[0], gc[1], gc[2]);
    // per dim: up to two frames (offset o of the local coordinate) that land;
    // scalars per (dim, slot) so nothing is indexed dynamically (no local memory)
    int nval[3], oa[3], ob[3], ga[3], gb[3];
    bool far = false;
#pragma unroll
    for (int d = 0; d < 3; d++) {
      int H, L;
      tile_local(g, gc[d], H, L);
      int xcode = load_code(a.xp, 3 * p + d, g.izipx);
      int vcode = load_code(a.vp, 3 * p + d, g.izipv);
      float vfd = a.vfield[3 * cell + d];
      // fast path: v = dec+vfield, P = dt_mid*v, deltax = P/4 in FP32 with bound Edx
      float dh = codec_decode_ff(a.cv, vcode).x;
      float vfa = __fadd_rn(dh, vfd);
      float Pf = __fmul_rn(dtm(a), vfa);
      float dxf = __fmul_rn(Pf, 0.25f);
      float Edx = 0.25f * (fabsf(dtm(a)) * (fabsf(dh) + fabsf(vfa)) * 1.2e-7f + fabsf(Pf) * 6.0e-8f);
      float offf = __fmul_rn(pos_off_f(xcode, g.izipx), g.izipx == 1 ? 1.0f / 256.0f : 1.0f / 65536.0f);
      nval[d] = 0;
      oa[d] = ob[d] = ga[d] = gb[d] = 0;
#pragma unroll
      for (int f = 0; f < 3; f++) {
        int o = f == 0 ? 0 : (f == 1 ? g.nt : -g.nt);
        int Ls = L + o;
        if (Ls < 1 - g.ncb || Ls > g.nt + g.ncb) continue;  // frame does not see this cell
        float xqf = __fadd_rn((float)(Ls - 1), offf);
        float sf = __fadd_rn(xqf, dxf);
        float Es = 1.25f * (Edx + (fabsf(xqf) + fabsf(sf)) * 6.0e-8f + 2.4e-7f * fabsf(sf)) + 1.0e-30f;
        float clo = ceilf(__fsub_rn(sf, Es)), chi = ceilf(__fadd_rn(sf, Es));
        int ig;
        if (clo == chi && !a.exact_only) {
          ig = (int)chi;
        } else {
          ig = dest_exact(a.cv, vcode, vfd, dtm(a), Ls, offf);
        }
        if (ig < 1 - 2 * g.ncb || ig > g.nt + 2 * g.ncb) {
          far = true;
          continue;
        }
        if (ig >= 1 && ig <= g.nt && nval[d] < 2) {
          if (nval[d] == 0) {
            oa[d] = o;
            ga[d] = ig;
          } else {
            ob[d] = o;
            gb[d] = ig;
          }
          nval[d]++;
          local_max = max(local_max, abs(ig - Ls));
        }
      }
    }
    if (far) atomicOr(&a.st->flags, 1);
    int ncopy = nval[0] * nval[1] * nval[2];
    if (ncopy == 0) {
      a.dest[p] = -1;
      a.doff[p] = 255;
      atomicAdd(&a.st->nlost, 1ull);
      continue;
    }
    for (int k = 0; k < ncopy; k++) {
      int sel[3] = {k % nval[0], (k / nval[0]) % nval[1], k / (nval[0] * nval[1])};
      int dg[3], fr = 0;
#pragma unroll
      for (int d = 0; d < 3; d++) {
        int H = (int)fdiv((uint32_t)gc[d], g.dnt);
        int o = sel[d] ? ob[d] : oa[d];
        int ig = sel[d] ? gb[d] : ga[d];
        // frame tile = H - o/nt (periodic in tiles); destination global coordinate
        int fo = o == 0 ? 0 : (o > 0 ? 1 : -1);
        int T = wrap1(H - fo, g.nnt);
        dg[d] = glob(g, T, ig);
      }
#pragma unroll
      for (int d = 2; d >= 0; d--) {
        int o = sel[d] ? ob[d] : oa[d];
        fr = 3 * fr + (o == 0 ? 1 : (o > 0 ? 2 : 0));
      }
      int32_t D = (int32_t)cell_id(g, dg[0], dg[1], dg[2]);
      if (k == 0) {
        a.dest[p] = D;
        a.dframe[p] = (uint8_t)fr;
        // offset of the source from the destination in the destination's frame
        int oc = 0;
        bool near = true;
#pragma unroll
        for (int d = 2; d >= 0; d--) {
          int H, L;
          tile_local(g, gc[d], H, L);
          int o = sel[d] ? ob[d] : oa[d], ig = sel[d] ? gb[d] : ga[d];
          int off = L + o - ig;
          near = near && off >= -1 && off <= 1;
          oc = 3 * oc + (off + 1);
        }
        a.doff[p] = near ? (uint8_t)oc : (uint8_t)255;
      } else {
        unsigned long long slot = atomicAdd(&a.st->ndup_list, 1ull);
        if ((int64_t)slot < a.xtra_cap) a.xtra[slot] = make_int4((int)p, D, -1, fr);
      }
    }
  }
  // block max of the displacement
  for (int o = 16; o > 0; o >>= 1) local_max = max(local_max, __shfl_xor_sync(0xffffffffu, local_max, o));
  if ((threadIdx.x & 31) == 0) atomicMax(&a.st->max_disp, local_max);
}

// vfield_new = vfield_new + vreal (update_particle.f90:72): the real(8) sum
// rounded to real(4), with vreal = decode + vfield(source) in real(8).  Fast
// path: the exact sum acc + dec + vfield as float-float, certified to round to
// the same float as the reference's two FP64 roundings followed by one FP32.
__device__ __forceinline__ float accumulate_vals(const UpdArgs& a, float acc, int vcode, float2 dd, float vfs) {
  float s1, e1, s2, e2;
  two_sum(acc, dd.x, s1, e1);
  two_sum(s1, vfs, s2, e2);
  float lo = __fadd_rn(__fadd_rn(e1, e2), dd.y);
  float margin = 1.25f * (fabsf(dd.x) * 4.0e-15f + (fabsf(e1) + fabsf(e2) + fabsf(dd.y)) * 1.2e-7f +
                          (fabsf(acc) + fabsf(dd.x) + fabsf(vfs)) * 2.3e-16f);
  float r;
  if (!a.exact_only && round_certified(s2, lo, margin, &r)) return r;
  return accumulate_exact(a.cv, vcode, vfs, acc);
}
__device__ __forceinline__ float accumulate_v(const UpdArgs& a, float acc, int64_t p, int d, int64_t S) {
  const int vcode = load_code(a.vp, 3 * p + d, a.g.izipv);
  return accumulate_vals(a, acc, vcode, codec_decode_ff(a.cv, vcode), a.vfield[3 * S + d]);
}

// vfield_new/(rhoce+weight_v) (update_particle.f90:81-83): the denominator
// cnt + (double)0.1f is exact in real(8); the quotient is rounded to real(8)
// and then to real(4).  Fast path: float-float quotient, certified as above.
__device__ __forceinline__ float vfield_quotient(float acc, uint32_t cnt, int exact_only) {
  float dhi, dlo;
  two_sum((float)cnt, 0.1f, dhi, dlo);  // (float)cnt exact below 2^24
  float q1 = __fdiv_rn(acc, dhi);
  float r1 = __fmaf_rn(-q1, dhi, acc);  // exact remainder of a correctly rounded quotient
  float lo = __fdiv_rn(__fsub_rn(r1, __fmul_rn(q1, dlo)), dhi);
  float margin = 1.25f * (fabsf(lo) * 3.6e-7f + fabsf(q1) * (fabsf(dlo / dhi) * fabsf(dlo / dhi) + 2.3e-16f));
  float r;
  if (!exact_only && cnt < (1u << 24) && round_certified(q1, lo, margin, &r)) return r;
  return quotient_exact(acc, cnt);
}

// U2 fast path, valid when every particle moved at most one cell and none
// landed in two frames (the usual step).  The rank of particle p in its
// destination D is the number of particles reaching D from the source cells
// D visits before p's cell, plus p's rank among the particles of its own cell
// bound for D.  Steps: per source cell, local ranks and 27 counts (one per
// neighbour it feeds); per destination, the counts in visit order turned into
// base ranks in place; after the scan, rank = base + local rank and the
// inverse permutation; per destination, vfield_new summed in rank order, i.e.
// the reference's visit order.
constexpr int NOFF = 27;

// one thread per particle: its rank among the earlier particles of its cell
// bound for the same neighbour (storage order); the last of them also writes
// that neighbour's count (the counts start at zero).  Cells denser than
// RL_MAX particles are listed for k_rank_dense (a block per cell).
constexpr int RL_MAX = 128;
constexpr int RD_THREADS = 256;

__global__ void k_rank_local(UpdArgs a) {
  if (a.st->max_disp > 1 || a.st->ndup_list != 0) {
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicOr(&a.st->flags, 8);  // not eligible
    return;
  }
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < a.np; p += (int64_t)gridDim.x * blockDim.x) {
    const int64_t S = a.pcell[p];
    const int64_t p0 = a.cstart[S], p1 = a.cstart[S + 1];
    if (p1 - p0 > RL_MAX) {  // the cell's first particle lists it
      if (p == p0) a.vdense[atomicAdd(&a.st->nrank_dense, 1u)] = (int32_t)S;
      continue;
    }
    const int o = a.doff[p];
    if (o == 255) {
      if (a.dest[p] >= 0) atomicOr(&a.st->flags, 4);  // moved farther than one cell
      continue;
    }
    int r = 0;
    bool last = true;
    for (int64_t q = p0; q < p1; q++) {
      if (a.doff[q] != o || q == p) continue;
      if (q < p) r++;
      else last = false;
    }
    a.lrank[p] = (uint16_t)r;
    if (last) a.offc[o * a.ncells + S] = (uint16_t)(r + 1);
  }
}

// The source cells k_rank_local listed (over RL_MAX particles), one block
// per cell: each particle's rank among the cell's earlier particles bound for
// the same neighbour and the 27 counts, as k_rank_local gives them.  The
// cell's particles go in chunks of RD_THREADS, in storage order: within a
// warp the rank is the count of lower lanes with the same neighbour
// (__match_any_sync), across the chunk's warps a table of per-warp counts,
// across chunks running counts.  A cell over 65535 particles (16-bit ranks)
// sends the step to the sort path.
__global__ void __launch_bounds__(RD_THREADS) k_rank_dense(UpdArgs a) {
  constexpr int NW = RD_THREADS / 32;
  __shared__ int wcnt[NW][NOFF];
  __shared__ int run[NOFF];
  const int n = (int)a.st->nrank_dense;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int it = blockIdx.x; it < n; it += gridDim.x) {
    const int64_t S = a.vdense[it];
    const int64_t p0 = a.cstart[S], p1 = a.cstart[S + 1];
    if (p1 - p0 > 65535) {
      if (threadIdx.x == 0) atomicOr(&a.st->flags, 4);
      continue;
    }
    for (int o = threadIdx.x; o < NOFF; o += blockDim.x) run[o] = 0;
    for (int64_t b = p0; b < p1; b += RD_THREADS) {
      for (int k = threadIdx.x; k < NW * NOFF; k += blockDim.x) (&wcnt[0][0])[k] = 0;
      __syncthreads();
      const int64_t p = b + threadIdx.x;
      int o = 255;
      if (p < p1) {
        o = a.doff[p];
        if (o == 255 && a.dest[p] >= 0) atomicOr(&a.st->flags, 4);  // moved farther than one cell
      }
      const unsigned peers = __match_any_sync(0xffffffffu, o);
      const int rw = __popc(peers & ((1u << lane) - 1u));
      if (o != 255 && rw == 0) wcnt[w][o] = __popc(peers);
      __syncthreads();
      if (o != 255) {
        int r = run[o] + rw;
        for (int v = 0; v < w; v++) r += wcnt[v][o];
        a.lrank[p] = (uint16_t)r;
      }
      __syncthreads();
      for (int k = threadIdx.x; k < NOFF; k += blockDim.x) {
        int s = 0;
        for (int v = 0; v < NW; v++) s += wcnt[v][k];
        run[k] += s;
      }
      __syncthreads();  // the table is read before the next chunk clears it
    }
    __syncthreads();
    for (int o = threadIdx.x; o < NOFF; o += blockDim.x)
      if (run[o]) a.offc[o * a.ncells + S] = (uint16_t)run[o];
    __syncthreads();
  }
}

// one thread per destination: the 27 counts it owns, read together, turned
// into base ranks in the destination's visit order, written back in place
__global__ void k_rank_base(UpdArgs a) {
  const Geo& g = a.g;
  if (a.st->flags & 12) return;
  for (int64_t D = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; D < a.ncells;
       D += (int64_t)gridDim.x * blockDim.x) {
    int dgc[3], T[3], Dl[3];
    cell_coords(g, D, dgc[0], dgc[1], dgc[2]);
#pragma unroll
    for (int d = 0; d < 3; d++) tile_local(g, dgc[d], T[d], Dl[d]);
    // source cells and their count of particles bound for D, in (dz, dy, dx) order
    uint32_t sid[NOFF];
    uint16_t c[NOFF];
#pragma unroll
    for (int dz = -1; dz <= 1; dz++) {
      int sz = glob(g, T[2], Dl[2] + dz);
#pragma unroll
      for (int dy = -1; dy <= 1; dy++) {
        int sy = glob(g, T[1], Dl[1] + dy);
#pragma unroll
        for (int dx = -1; dx <= 1; dx++) {
          const int o = (dx + 1) + 3 * (dy + 1) + 9 * (dz + 1);
          sid[o] = (uint32_t)cell_id(g, glob(g, T[0], Dl[0] + dx), sy, sz);
          c[o] = a.offc[o * a.ncells + sid[o]];
        }
      }
    }
    // the three source z-slabs in visit order: by (layer, k), layer=(k+ncb-1) mod nlayer
    int key[3];
#pragma unroll
    for (int i = 0; i < 3; i++) {
      int kl = Dl[2] + i - 1;
      key[i] = ((kl + g.ncb - 1) % nlay(a)) * 4096 + kl + 8;
    }
    int zo[3] = {0, 1, 2};  // slab index dz+1
    if (key[1] < key[0]) { int t = key[0]; key[0] = key[1]; key[1] = t; t = zo[0]; zo[0] = zo[1]; zo[1] = t; }
    if (key[2] < key[1]) { int t = key[1]; key[1] = key[2]; key[2] = t; t = zo[1]; zo[1] = zo[2]; zo[2] = t; }
    if (key[1] < key[0]) { int t = key[0]; key[0] = key[1]; key[1] = t; t = zo[0]; zo[0] = zo[1]; zo[1] = t; }
    uint32_t base = 0, bz[3];
    uint32_t sum[3];
#pragma unroll
    for (int z = 0; z < 3; z++) {
      uint32_t s = 0;
#pragma unroll
      for (int k = 0; k < 9; k++) s += c[9 * z + k];
      sum[z] = s;
    }
    for (int i = 0; i < 3; i++) {
      bz[zo[i]] = base;
      base += sum[zo[i]];
    }
    if (base > 0xffffu) atomicOr(&a.st->flags, 4);
#pragma unroll
    for (int z = 0; z < 3; z++) {
      uint32_t b = bz[z];
#pragma unroll
      for (int k = 0; k < 9; k++) {
        const int o = 9 * z + k;
        a.offc[o * a.ncells + sid[o]] = (uint16_t)b;
        b += c[o];
      }
    }
    a.cnt_new[D] = (int32_t)base;
  }
}

__global__ void k_rank_place(UpdArgs a) {
  if (a.sd && counting_failed(a)) return;
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < a.np; p += (int64_t)gridDim.x * blockDim.x) {
    int32_t D = a.dest[p];
    if (D < 0) continue;
    uint32_t r = (uint32_t)a.offc[a.doff[p] * a.ncells + a.pcell[p]] + a.lrank[p];
    a.rank[p] = r;
    if (r < (uint32_t)a.cnt_new[D]) a.perm[a.cstart_new[D] + r] = (int32_t)p;
    else atomicOr(&a.st->flags, 2);
  }
}

// a cell over VF_DENSE particles goes to k_vfield_dense: one thread summing
// hundreds of particles in rank order would set the kernel's tail.  The
// thread path loads VF_BATCH particles' codes, decoded values and source
// means ahead of their (sequential) sums, so the loads of a batch overlap.
constexpr uint32_t VF_DENSE = 256;
constexpr uint32_t VF_BATCH = 4;
__global__ void k_vfield_new(UpdArgs a) {
  if (a.sd && counting_failed(a)) return;
  for (int64_t D = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; D < a.ncells;
       D += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t cnt = (uint32_t)a.cnt_new[D];
    if (cnt > VF_DENSE) {
      a.vdense[atomicAdd(&a.st->ndense, 1u)] = (int32_t)D;
      continue;
    }
    float acc[3];
#pragma unroll
    for (int d = 0; d < 3; d++) acc[d] = __fmul_rn(a.vfield[3 * D + d], 0.1f);  // vfield*weight_v
    const int64_t i0 = a.cstart_new[D];
    for (uint32_t i = 0; i < cnt; i += VF_BATCH) {
      int64_t pb[VF_BATCH], Sb[VF_BATCH];
      int code[VF_BATCH][3];
      float vfs[VF_BATCH][3];
      float2 dd[VF_BATCH][3];
#pragma unroll
      for (uint32_t j = 0; j < VF_BATCH; j++) pb[j] = i + j < cnt ? a.perm[i0 + i + j] : a.perm[i0 + i];
#pragma unroll
      for (uint32_t j = 0; j < VF_BATCH; j++) {
        Sb[j] = a.pcell[pb[j]];
#pragma unroll
        for (int d = 0; d < 3; d++) code[j][d] = load_code(a.vp, 3 * pb[j] + d, a.g.izipv);
      }
#pragma unroll
      for (uint32_t j = 0; j < VF_BATCH; j++)
#pragma unroll
        for (int d = 0; d < 3; d++) {
          vfs[j][d] = a.vfield[3 * Sb[j] + d];
          dd[j][d] = codec_decode_ff(a.cv, code[j][d]);
        }
#pragma unroll
      for (uint32_t j = 0; j < VF_BATCH; j++)
        if (i + j < cnt)
#pragma unroll
          for (int d = 0; d < 3; d++) acc[d] = accumulate_vals(a, acc[d], code[j][d], dd[j][d], vfs[j][d]);
    }
#pragma unroll
    for (int d = 0; d < 3; d++) a.vfield_new[3 * D + d] = vfield_quotient(acc[d], cnt, a.exact_only);
  }
}

// vfield_new of the listed dense cells, one warp per cell: the lanes load 32
// particles' codes, decoded values and source-cell means at a time (all
// independent), then lanes 0-2 -- one per component -- run the reference's
// sequential real(4) sum over them in rank order, the same arithmetic as
// k_vfield_new's thread
__global__ void __launch_bounds__(128) k_vfield_dense(UpdArgs a) {
  if (a.sd && counting_failed(a)) return;
  __shared__ float2 sdd[4][32][3];
  __shared__ float svf[4][32][3];
  __shared__ int scode[4][32][3];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t nw = (int64_t)gridDim.x * (blockDim.x >> 5);
  const uint32_t n = *(volatile unsigned int*)&a.st->ndense;
  for (int64_t it = blockIdx.x * (int64_t)(blockDim.x >> 5) + w; it < (int64_t)n; it += nw) {
    const int64_t D = a.vdense[it];
    const uint32_t cnt = (uint32_t)a.cnt_new[D];
    const int64_t i0 = a.cstart_new[D];
    float acc = lane < 3 ? __fmul_rn(a.vfield[3 * D + lane], 0.1f) : 0.f;  // vfield*weight_v
    for (uint32_t j0 = 0; j0 < cnt; j0 += 32) {
      const uint32_t m = min(32u, cnt - j0);
      if ((uint32_t)lane < m) {
        const int64_t p = a.perm[i0 + j0 + lane];
        const int64_t S = a.pcell[p];
#pragma unroll
        for (int d = 0; d < 3; d++) {
          const int vcode = load_code(a.vp, 3 * p + d, a.g.izipv);
          scode[w][lane][d] = vcode;
          sdd[w][lane][d] = codec_decode_ff(a.cv, vcode);
          svf[w][lane][d] = a.vfield[3 * S + d];
        }
      }
      __syncwarp();
      if (lane < 3)
        for (uint32_t j = 0; j < m; j++) acc = accumulate_vals(a, acc, scode[w][j][lane], sdd[w][j][lane], svf[w][j][lane]);
      __syncwarp();
    }
    if (lane < 3) a.vfield_new[3 * D + lane] = vfield_quotient(acc, cnt, a.exact_only);
  }
}

// U2: one thread per destination cell walks the sources in visit order.
__global__ void k_rank(UpdArgs a) {
  if (a.sd && !counting_failed(a)) return;
  const Geo& g = a.g;
  int R = min(a.st->max_disp, 2 * g.ncb);
  int64_t nx = (int64_t)(a.st->ndup_list < (unsigned long long)a.xtra_cap ? a.st->ndup_list : (unsigned long long)a.xtra_cap);
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t D = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; D < a.ncells; D += stride) {
    int dgc[3];
    cell_coords(g, D, dgc[0], dgc[1], dgc[2]);
    int T[3], Dl[3];
    for (int d = 0; d < 3; d++) {
      tile_local(g, dgc[d], T[d], Dl[d]);
    }
    // source z offsets sorted by (layer, k): layer = (k+ncb-1) mod nlayer
    int dz[2 * 16 + 1];
    int nz = 0;
    for (int o = -R; o <= R; o++) {
      int kl = Dl[2] + o;
      if (kl < 1 - g.ncb || kl > g.nt + g.ncb) continue;
      int lay = (kl + g.ncb - 1) % nlay(a);
      int pos = nz++;
      while (pos > 0) {
        int ko = Dl[2] + dz[pos - 1];
        int lo = (ko + g.ncb - 1) % nlay(a);
        if (lo > lay || (lo == lay && ko > kl)) {
          dz[pos] = dz[pos - 1];
          pos--;
        } else {
          break;
        }
      }
      dz[pos] = o;
    }
    // vfield_new=vfield*weight_v: the product of two floats is exact in real(8),
    // so its real(4) rounding is the FP32 product
    float acc[3];
    for (int d = 0; d < 3; d++) acc[d] = __fmul_rn(a.vfield[3 * D + d], 0.1f);
    uint32_t cnt = 0;
    for (int iz = 0; iz < nz; iz++) {
      int kl = Dl[2] + dz[iz];
      int sz = glob(g, T[2], kl);
      // frame offset (in tiles) at which this destination tile sees the source:
      // local coordinate kl vs the source's own tile-local coordinate
      int fz = frame_code(g, kl, sz);
      for (int jl = Dl[1] - R; jl <= Dl[1] + R; jl++) {
        if (jl < 1 - g.ncb || jl > g.nt + g.ncb) continue;
        int sy = glob(g, T[1], jl);
        int fy = frame_code(g, jl, sy);
        for (int il = Dl[0] - R; il <= Dl[0] + R; il++) {
          if (il < 1 - g.ncb || il > g.nt + g.ncb) continue;
          int sx = glob(g, T[0], il);
          int fx = frame_code(g, il, sx);
          uint8_t fr = (uint8_t)(fx + 3 * fy + 9 * fz);
          int64_t S = cell_id(g, sx, sy, sz);
          int64_t p0 = a.cstart[S], p1 = a.cstart[S + 1];
          for (int64_t p = p0; p < p1; p++) {
            bool hit = a.dest[p] == (int32_t)D && a.dframe[p] == fr;
            int64_t xi = -1;
            if (!hit && nx > 0) {
              for (int64_t e = 0; e < nx; e++)
                if (a.xtra[e].x == (int)p && a.xtra[e].y == (int)D && a.xtra[e].w == (int)fr) xi = e;
            }
            if (!hit && xi < 0) continue;
            if (hit)
              a.rank[p] = cnt;
            else
              a.xtra[xi].z = (int)cnt;
            cnt++;
            for (int d = 0; d < 3; d++) acc[d] = accumulate_v(a, acc[d], p, d, S);
          }
        }
      }
    }
    a.cnt_new[D] = (int32_t)cnt;
    for (int d = 0; d < 3; d++) a.vfield_new[3 * D + d] = vfield_quotient(acc[d], cnt, a.exact_only);
  }
}

// particle p, landed in cell D, written at index idx of the new arrays
__device__ __forceinline__ void write_particle_at(const UpdArgs& a, int64_t p, int32_t D, int64_t idx) {
  const Geo& g = a.g;
  int64_t cell = a.pcell[p];
  // nint(dt_mid*vreal/(x_resolution*ncell)): the divisor is a power of two
  float scale = g.izipx == 1 ? 64.0f : 16384.0f;
  for (int d = 0; d < 3; d++) {
    int vcode = load_code(a.vp, 3 * p + d, g.izipv);
    float vfd = a.vfield[3 * cell + d];
    float vbar = a.vfield_new[3 * (int64_t)D + d];
    float2 dd = codec_decode_ff(a.cv, vcode);
    // drift in code units: FP32 estimate of dt_mid*(dec+vfield)*scale with its bound
    float vfa = __fadd_rn(dd.x, vfd);
    float Pf = __fmul_rn(dtm(a), vfa);
    float EP = scale * 1.25f * (fabsf(dtm(a)) * (fabsf(dd.x) + fabsf(vfa)) * 1.2e-7f + fabsf(Pf) * 6.0e-8f);
    long long dx;
    if (a.exact_only || !nint_certified(__fmul_rn(Pf, scale), EP, &dx)) {
      double v = __dadd_rn(codec_decode(a.cv, vcode), (double)vfd);
      dx = llround(__dmul_rn(__dmul_rn((double)dtm(a), v), (double)scale));
    }
    long long x = load_code(a.xp, 3 * p + d, g.izipx);
    store_code(a.xp_new, 3 * idx + d, g.izipx, x + dx);
    // vp = code of vreal - vfield_new (update_particle.f90:116-117)
    float w, ew;
    two_sum(vfd, -vbar, w, ew);
    float Vf = __fadd_rn(dd.x, w);
    float E = 1.25f * ((fabsf(dd.x) + fabsf(Vf)) * 6.0e-8f + fabsf(ew) +
                       (fabsf(dd.x) + fabsf(vfd) + fabsf(vbar)) * 2.3e-16f);
    long long ab = f2d_bits(Vf) & 0x7fffffffffffffffLL, n = 0, code;
    if (!a.exact_only && certify_abs(ab, E, a.cv, &n)) {
      code = Vf < 0.f ? -n : n;
    } else {
      double v = __dadd_rn(codec_decode(a.cv, vcode), (double)vfd);
      code = codec_encode(a.cv, __dsub_rn(v, (double)vbar));
    }
    store_code(a.vp_new, 3 * idx + d, g.izipv, code);
  }
  a.pid_new[idx] = a.pid[p];
  a.pcell_new[idx] = D;
}

__device__ __forceinline__ void write_particle(const UpdArgs& a, int64_t p, int32_t D, uint32_t r) {
  if (D < 0 || (int64_t)D >= a.ncells || r >= (uint32_t)a.cnt_new[D]) {
    atomicOr(&a.st->flags, 2);  // rank not assigned: never write outside the new arrays
    return;
  }
  write_particle_at(a, p, D, a.cstart_new[D] + r);
}

// U2, general path: the rank of a landing (a particle's primary destination,
// or an extra copy's) is its position among the landings in its destination
// cell ordered by the reference's visit order, and the new disjoint order is
// the cells in storage order with their particles by rank.  So one sort of
// all landings by
//   (destination cell, layer of the source's z in the destination tile's
//    frame, source offsets z, y, x from the destination, index in the
//    source cell)
// yields the new order itself: position = cstart_new[D] + rank.  The fields
// are as wide as this step needs: offsets + R in ob bits (|offset| <= R, the
// largest displacement), the layer in bits(nlayer), the index in the source
// cell in the lb bits left below (a landing that does not fit flags itself
// and the walker takes over).  Without extra copies the sort skips the index
// bits: the radix sort is stable and the primaries enter in storage order,
// which within a source cell is the index order.
inline int bits_for(int64_t n) {  // smallest b with 2^b >= n
  int b = 0;
  while (((int64_t)1 << b) < n) b++;
  return b;
}

__global__ void k_sort_keys(UpdArgs a, uint64_t* __restrict__ keys, int32_t* __restrict__ vals, int64_t nx, int lb,
                            int ob, int R, int vb) {
  const Geo& g = a.g;
  const int64_t n = a.np + nx;
  const uint64_t lmax = (uint64_t)1 << lb;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    int64_t p;
    int32_t D;
    int fr;
    if (i < a.np) {
      p = i;
      D = a.dest[p];
      fr = a.dframe[p];
    } else {
      const int4 x = a.xtra[i - a.np];
      p = x.x;
      D = x.y;
      fr = x.w;
    }
    vals[i] = (int32_t)i;
    if (D < 0 || (int64_t)D >= a.ncells) {  // lost: after every landing
      keys[i] = ~0ull;
      continue;
    }
    const int64_t S = a.pcell[p];
    const uint64_t l = (uint64_t)(p - a.cstart[S]);
    int sg[3], dg[3];
    cell_coords(g, S, sg[0], sg[1], sg[2]);
    cell_coords(g, D, dg[0], dg[1], dg[2]);
    uint64_t visit = 0;
    int layer = 0;
    bool bad = l >= lmax;
    for (int d = 2; d >= 0; d--) {
      int T, L, TD, DL;
      tile_local(g, sg[d], T, L);
      tile_local(g, dg[d], TD, DL);
      const int digit = d == 2 ? fr / 9 : (d == 1 ? (fr / 3) % 3 : fr % 3);
      const int Ls = L + (digit - 1) * g.nt;  // the source in the destination tile's frame
      const int off = Ls - DL;
      bad = bad || off < -R || off > R;
      if (d == 2) layer = (Ls + g.ncb - 1) % nlay(a);
      visit = (visit << ob) | (uint64_t)((off + R) & ((1 << ob) - 1));
    }
    if (bad) atomicOr(&a.st->flags, 64);  // does not fit the key: the walker takes over
    visit |= (uint64_t)layer << (3 * ob);
    keys[i] = ((uint64_t)D << (vb + lb)) | (visit << lb) | (l & (lmax - 1));
    atomicAdd(&a.cnt_new[D], 1);
  }
}

// the inverse permutation (new index -> particle) from the sorted landings
__global__ void k_sort_place(UpdArgs a, const int32_t* __restrict__ vals, int64_t n_new) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n_new; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t id = vals[i];
    a.perm[i] = id < a.np ? (int32_t)id : a.xtra[id - a.np].x;
  }
}

// U3 on the sort path: one thread per new index writes the particle that
// lands there (coalesced writes; the reads stay within a few cells of the
// destination, which L2 holds)
__global__ void k_sort_gather(UpdArgs a, const uint64_t* __restrict__ keys, int64_t n_new, int shift) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n_new; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t D = (int64_t)(keys[i] >> shift);
    if (D >= a.ncells || i < a.cstart_new[D] || i >= a.cstart_new[D + 1]) {
      atomicOr(&a.st->flags, 2);
      continue;
    }
    write_particle_at(a, a.perm[i], (int32_t)D, i);
  }
}

// U3: scatter every primary copy to its place in the new disjoint order.
__global__ void k_scatter(UpdArgs a) {
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < a.np; p += stride) {
    int32_t D = a.dest[p];
    if (D >= 0) write_particle(a, p, D, a.rank[p]);
  }
}

__global__ void k_scatter_xtra(UpdArgs a) {
  int64_t nx = (int64_t)(a.st->ndup_list < (unsigned long long)a.xtra_cap ? a.st->ndup_list : (unsigned long long)a.xtra_cap);
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < nx; e += (int64_t)gridDim.x * blockDim.x)
    write_particle(a, a.xtra[e].x, a.xtra[e].y, (uint32_t)a.xtra[e].z);
}

__device__ __forceinline__ void ff_add(float& hi, float& lo, float x, float xlo) {
  float s, e;
  two_sum(hi, x, s, e);
  e = __fadd_rn(e, __fadd_rn(lo, xlo));
  two_sum(s, e, hi, lo);
}

// sigma_v sums of the new state (update_particle.f90:172-196): per-block FP64
// partials in a fixed partition, summed in block order on the host.
__global__ void k_sigma(const void* __restrict__ vp, const int32_t* __restrict__ pcell, const float* __restrict__ vfield,
                        int64_t np, int64_t ncells, const float2* __restrict__ dech, int nvbin, int izipv,
                        double* __restrict__ part) {
  __shared__ double s[3][32];
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  int64_t t0 = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  // per-thread float-float accumulators (exact products by FMA), one FP64
  // combine per thread: FP64-accurate sums without FP64 per element
  float ch = 0.f, cl = 0.f, rh = 0.f, rl = 0.f, sh = 0.f, sl = 0.f;
  for (int64_t c = t0; c < ncells; c += stride) {
    float a0 = vfield[3 * c], a1 = vfield[3 * c + 1], a2 = vfield[3 * c + 2];
    float q = __fadd_rn(__fadd_rn(__fmul_rn(a0, a0), __fmul_rn(a1, a1)), __fmul_rn(a2, a2));
    ff_add(ch, cl, q, 0.f);
  }
  for (int64_t p = t0; p < np; p += stride) {
    int64_t c = pcell[p];
    if (c < 0 || c >= ncells) continue;
    for (int d = 0; d < 3; d++) {
      float2 v = __ldg(dech + load_code(vp, 3 * p + d, izipv) + nvbin / 2);
      float p2 = __fmul_rn(v.x, v.x);
      ff_add(rh, rl, p2, __fmaf_rn(v.x, v.x, -p2) + 2.f * v.x * v.y);
      float w, ew;
      two_sum(v.x, vfield[3 * c + d], w, ew);
      ew += v.y;
      float q2 = __fmul_rn(w, w);
      ff_add(sh, sl, q2, __fmaf_rn(w, w, -q2) + 2.f * w * ew);
    }
  }
  double sc = (double)ch + (double)cl, sr = (double)rh + (double)rl, ss = (double)sh + (double)sl;
  for (int o = 16; o > 0; o >>= 1) {
    sc += __shfl_xor_sync(0xffffffffu, sc, o);
    sr += __shfl_xor_sync(0xffffffffu, sr, o);
    ss += __shfl_xor_sync(0xffffffffu, ss, o);
  }
  int w = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0) {
    s[0][w] = sc;
    s[1][w] = sr;
    s[2][w] = ss;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double t[3] = {0, 0, 0};
    for (int i = 0; i < (int)(blockDim.x >> 5); i++)
      for (int k = 0; k < 3; k++) t[k] += s[k][i];
    for (int k = 0; k < 3; k++) part[3 * blockIdx.x + k] = t[k];
  }
}

// graph mode: sigma_vi_new from the block partials on the device, with the
// host path's arithmetic (the same summation order, correctly rounded sqrt
// and division), its vcoef for the encode estimate, and the sums for the host
__global__ void k_sigma_final(const double* __restrict__ part, int nb, double npg, StepDev* sd, StepOut* so) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  double s[3] = {0.0, 0.0, 0.0};
  for (int b = 0; b < nb; b++)
    for (int t = 0; t < 3; t++) s[t] += part[3 * b + t];
  const double std_res = sqrt(s[1] / npg);
  const float sn = (float)(std_res / (double)sqrtf(3.0f));  // update_particle.f90:224
  sd->sigma_new = sn;
  sd->cf_new = sn > 0.f ? (float)vcoef(sn) : 0.f;
  if (so) {
    for (int t = 0; t < 3; t++) so->sums[t] = s[t];
    so->sigma_new = sn;
  }
}

}  // namespace

// update_x inside a captured graph (cube_batch_*): the step scalars come from
// c->sd, both rank paths are launched and each decides on the device whether
// it runs, the extra-copy list is walked up to its device count, and
// sigma_vi_new and its codec tables (slot 1) are computed on the device.  The
// particle count of an image never changes (the box is periodic), so every
// grid is fixed.  Stats land in c->sout->upd; the host checks them after the
// step.
static int update_x_graph(cube_ctx* c) {
  Geo g = make_geo(c);
  int k = c->cur, kn = 1 - k;
  CodecView cv;
  cube_codec_view_dev(c, 0, &c->sd->h.cf_vi, &cv);
  CUBE_CUDA(c, cudaMemsetAsync(c->dstats, 0, sizeof(DevStats), c->stream));
  UpdArgs a{};
  a.g = g;
  a.np = c->np;
  a.ncells = c->ncells;
  a.dt_mid = 0.f;
  a.nlayer = 1;
  a.sd = c->sd;
  a.xp = c->xp[k];
  a.vp = c->vp[k];
  a.pid = c->pid[k];
  a.pcell = c->pcell[k];
  a.vfield = c->vfield[k];
  a.cstart = c->cstart[k];
  a.cv = cv;
  a.exact_only = c->opt_exact_kicks;
  a.dest = c->dest;
  a.dframe = c->dframe;
  a.doff = c->doff;
  a.lrank = c->lrank;
  a.offc = c->offc;
  a.perm = c->perm;
  a.rank = c->rank;
  a.xtra = c->xtra;
  a.xtra_cap = c->xtra_cap;
  a.st = c->dstats;
  a.cnt_new = c->rhoc[kn];
  a.vfield_new = c->vfield[kn];
  a.cstart_new = c->cstart[kn];
  a.xp_new = c->xp[kn];
  a.vp_new = c->vp[kn];
  a.pid_new = c->pid[kn];
  a.pcell_new = c->pcell[kn];
  a.vdense = c->vdense;
  const int B = 256;
  cudaStream_t s = c->stream;
  CUBE_CUDA(c, cudaMemsetAsync(c->rank, 0xFF, 4 * (size_t)c->np, s));
  k_dest<<<cube_grid(c->np, B), B, 0, s>>>(a);
  CUBE_CUDA(c, cudaMemsetAsync(c->offc, 0, sizeof(uint16_t) * NOFF * (size_t)c->ncells, s));
  k_rank_local<<<cube_grid(c->np, 256), 256, 0, s>>>(a);
  k_rank_dense<<<cube_grid((int64_t)1 << 40, 1, 4), RD_THREADS, 0, s>>>(a);
  k_rank_base<<<cube_grid(c->ncells, 256), 256, 0, s>>>(a);
  k_rank<<<cube_grid(c->ncells, 128, 32), 128, 0, s>>>(a);
  CUBE_CUDA(c, cudaGetLastError());
  int r = cube_scan_counts(c, c->rhoc[kn], c->cstart[kn], c->ncells);
  if (r) return r;
  k_rank_place<<<cube_grid(c->np, B), B, 0, s>>>(a);
  k_vfield_new<<<cube_grid(c->ncells, 128, 32), 128, 0, s>>>(a);
  k_vfield_dense<<<cube_grid((int64_t)1 << 40, 1, 16), 128, 0, s>>>(a);
  k_scatter<<<cube_grid(c->np, B), B, 0, s>>>(a);
  k_scatter_xtra<<<cube_grid(c->xtra_cap, B, 2), B, 0, s>>>(a);
  const int nb = c->red_blocks;
  k_sigma<<<nb, 256, 0, s>>>(c->vp[kn], c->pcell[kn], c->vfield[kn], c->np, c->ncells, cv.dech, c->nvbin, c->p.izipv,
                             c->red_tmp);
  const double npg = (double)(c->npglobal > 0 ? c->npglobal : c->np);
  k_sigma_final<<<1, 32, 0, s>>>(c->red_tmp, nb, npg, c->sd, c->sout);
  CUBE_CUDA(c, cudaGetLastError());
  CUBE_CUDA(c, cudaMemcpyAsync(&c->sout->upd, c->dstats, sizeof(DevStats), cudaMemcpyDeviceToDevice, s));
  r = cube_codec_build_dev(c, 1, &c->sd->sigma_new);
  if (r) return r;
  c->cur = kn;
  c->rank_walked = 0;
  return CUBE_OK;
}

int cube_update_x_impl(cube_ctx* c, float dt_old, float dt, float vz_max, cube_stats* st) {
  if (c->graph_mode) return update_x_graph(c);
  Geo g = make_geo(c);
  int k = c->cur, kn = 1 - k;
  float dt_mid = (dt_old + dt) / 2.0f;  // update_particle.f90:32
  // nlayer=2*ceiling(dt_mid*sim%vz_max/ncell)+1 in real(4) (update_particle.f90:37)
  volatile float q = dt_mid * vz_max;
  volatile float q2 = q / (float)c->p.ncell;
  int nlayer = 2 * (int)std::ceil((double)q2) + 1;
  if (nlayer < 1) nlayer = 1;
  CodecView cv;
  int r = cube_codec_pair(c, c->sigma_vi, c->sigma_vi, &cv, nullptr);
  if (r) return r;
  CUBE_CUDA(c, cudaMemsetAsync(c->dstats, 0, sizeof(DevStats), c->stream));
  UpdArgs a{};
  a.g = g;
  a.np = c->np;
  a.ncells = c->ncells;
  a.dt_mid = dt_mid;
  a.nlayer = nlayer;
  a.xp = c->xp[k];
  a.vp = c->vp[k];
  a.pid = c->pid[k];
  a.pcell = c->pcell[k];
  a.vfield = c->vfield[k];
  a.cstart = c->cstart[k];
  a.cv = cv;
  a.exact_only = c->opt_exact_kicks;
  a.dest = c->dest;
  a.dframe = c->dframe;
  a.doff = c->doff;
  a.lrank = c->lrank;
  a.offc = c->offc;
  a.perm = c->perm;
  a.rank = c->rank;
  a.xtra = c->xtra;
  a.xtra_cap = c->xtra_cap;
  a.st = c->dstats;
  a.cnt_new = c->rhoc[kn];
  a.vfield_new = c->vfield[kn];
  a.cstart_new = c->cstart[kn];
  a.xp_new = c->xp[kn];
  a.vp_new = c->vp[kn];
  a.pid_new = c->pid[kn];
  a.pcell_new = c->pcell[kn];
  a.vdense = c->vdense;
  const int B = 256;
  CUBE_CUDA(c, cudaMemsetAsync(c->rank, 0xFF, 4 * (size_t)c->np, c->stream));  // "no rank" sentinel
  cube_phase_begin(c, PH_UPD_DEST);
  if (c->xv_pending && c->up_np == c->np) {
    // a pending cube_upload_begin: take xp and vp piece by piece as they land
    for (int i = 0; i < cube_ctx::UP_PIECES; i++) {
      UpdArgs ap = a;
      ap.p_lo = c->np * i / cube_ctx::UP_PIECES;
      ap.np = c->np * (i + 1) / cube_ctx::UP_PIECES;
      CUBE_CUDA(c, cudaStreamWaitEvent(c->stream, c->ev_xv[i], 0));
      if (ap.np > ap.p_lo) k_dest<<<cube_grid(ap.np - ap.p_lo, B), B, 0, c->stream>>>(ap);
    }
    c->xv_pending = false;  // pid (the last piece) is joined before the scatter
  } else {
    if ((r = cube_upload_join(c))) return r;
    k_dest<<<cube_grid(c->np, B), B, 0, c->stream>>>(a);
  }
  cube_phase_end(c, PH_UPD_DEST);
  // ranks: the counting path (its kernels check their own eligibility on the
  // device and flag it), else the sort of all landings; the visit-order
  // walker on request, or when a landing does not fit the sort key
  enum { COUNT = 0, WALK = 1, SORT = 2 };
  int path = c->opt_rank_walk;
  int64_t np_new = 0;
  auto walk = [&]() -> int {
    cube_phase_begin(c, PH_UPD_RANK);
    k_rank<<<cube_grid(c->ncells, 128, 32), 128, 0, c->stream>>>(a);
    cube_phase_end(c, PH_UPD_RANK);
    CUBE_CUDA(c, cudaGetLastError());
    return CUBE_OK;
  };
  auto scan = [&]() -> int {
    cube_phase_begin(c, PH_UPD_SCAN);
    int rr = cube_scan_counts(c, c->rhoc[kn], c->cstart[kn], c->ncells);
    cube_phase_end(c, PH_UPD_SCAN);
    if (rr) return rr;
    CUBE_CUDA(c, cudaMemcpyAsync(&np_new, c->cstart[kn] + c->ncells, 8, cudaMemcpyDeviceToHost, c->stream));
    return cube_stats_fetch(c);
  };
  if (path == COUNT) {
    cube_phase_begin(c, PH_UPD_RANK);
    CUBE_CUDA(c, cudaMemsetAsync(c->offc, 0, sizeof(uint16_t) * NOFF * (size_t)c->ncells, c->stream));
    k_rank_local<<<cube_grid(c->np, 256), 256, 0, c->stream>>>(a);
    k_rank_dense<<<cube_grid((int64_t)1 << 40, 1, 4), RD_THREADS, 0, c->stream>>>(a);
    k_rank_base<<<cube_grid(c->ncells, 256), 256, 0, c->stream>>>(a);
    cube_phase_end(c, PH_UPD_RANK);
    CUBE_CUDA(c, cudaGetLastError());
    if ((r = scan())) return r;
    if (c->hstats->flags & 12) path = SORT;  // counting path not applicable
  } else if (path == WALK) {
    if ((r = walk()) || (r = scan())) return r;
  } else {
    if ((r = cube_stats_fetch(c))) return r;
  }
  if (c->hstats->flags & 1) return cube_fail(c, CUBE_ERR_DISPLACEMENT, "a particle left the double-buffer tile");
  if ((int64_t)c->hstats->ndup_list > c->xtra_cap)
    return cube_fail(c, CUBE_ERR_TILE_OVERFLOW, "extra-copy list overflow");
  int db = 0;
  uint64_t* skeys = nullptr;
  if (path == SORT) {
    const int64_t nx = (int64_t)c->hstats->ndup_list;
    const int R = std::max(c->hstats->max_disp, 1);
    const int ob = bits_for(2 * R + 1), vb = bits_for(nlayer) + 3 * ob;
    db = bits_for(c->ncells);
    const int lb = 64 - db - vb;
    if (lb < 8) return cube_fail(c, CUBE_ERR_ARG, "too many cells for the re-sort key");
    CUBE_CUDA(c, cudaMemsetAsync(&c->dstats->flags, 0, sizeof(int), c->stream));
    cube_phase_begin(c, PH_UPD_RANK);
    CUBE_CUDA(c, cudaMemsetAsync(c->rhoc[kn], 0, 4 * (size_t)c->ncells, c->stream));
    uint64_t* keys = c->skey[0];
    int32_t* vals = c->sval[0];
    if ((r = cube_sort_pairs(c, 0, 0, 64, &keys, &vals))) return r;  // buffers
    k_sort_keys<<<cube_grid(c->np + nx, 256), 256, 0, c->stream>>>(a, keys, vals, nx, lb, ob, R, vb);
    CUBE_CUDA(c, cudaGetLastError());
    if ((r = cube_sort_pairs(c, c->np + nx, nx ? 0 : lb, 64, &keys, &vals))) return r;
    cube_phase_end(c, PH_UPD_RANK);
    if ((r = scan())) return r;
    if (c->hstats->flags & 64) {  // a landing did not fit the key
      CUBE_CUDA(c, cudaMemsetAsync(&c->dstats->flags, 0, sizeof(int), c->stream));
      path = WALK;
      if ((r = walk()) || (r = scan())) return r;
    } else {
      cube_phase_begin(c, PH_UPD_PLACE);
      k_sort_place<<<cube_grid(np_new, 256), 256, 0, c->stream>>>(a, vals, np_new);
      cube_phase_end(c, PH_UPD_PLACE);
      CUBE_CUDA(c, cudaGetLastError());
      skeys = keys;
    }
  }
  c->rank_walked = path;
  DevStats hs = *c->hstats;
  if (np_new > c->p.np_max)
    return cube_fail(c, CUBE_ERR_IMAGE_OVERFLOW, "new particle count exceeds np_max");
  if (path != WALK) {
    cube_phase_begin(c, PH_UPD_PLACE);
    if (path == COUNT) k_rank_place<<<cube_grid(c->np, B), B, 0, c->stream>>>(a);
    k_vfield_new<<<cube_grid(c->ncells, 128, 32), 128, 0, c->stream>>>(a);
    k_vfield_dense<<<cube_grid((int64_t)1 << 40, 1, 16), 128, 0, c->stream>>>(a);
    cube_phase_end(c, PH_UPD_PLACE);
    CUBE_CUDA(c, cudaGetLastError());
  }
  r = cube_pid_join(c);  // a deferred pid upload lands before the scatter reads it
  if (r) return r;
  cube_phase_begin(c, PH_UPD_SCATTER);
  if (skeys) {
    k_sort_gather<<<cube_grid(np_new, B), B, 0, c->stream>>>(a, skeys, np_new, 64 - db);
  } else {
    k_scatter<<<cube_grid(c->np, B), B, 0, c->stream>>>(a);
    if (hs.ndup_list) k_scatter_xtra<<<cube_grid((int64_t)hs.ndup_list, B), B, 0, c->stream>>>(a);
  }
  cube_phase_end(c, PH_UPD_SCATTER);
  CUBE_CUDA(c, cudaGetLastError());
  // sigma statistics of the new state (decoded with sigma_vi)
  int nb = c->red_blocks;
  cube_phase_begin(c, PH_UPD_SIGMA);
  k_sigma<<<nb, 256, 0, c->stream>>>(c->vp[kn], c->pcell[kn], c->vfield[kn], np_new, c->ncells, cv.dech,
                                      c->nvbin, c->p.izipv, c->red_tmp);
  cube_phase_end(c, PH_UPD_SIGMA);
  CUBE_CUDA(c, cudaGetLastError());
  std::vector<double> part(3 * (size_t)nb);
  CUBE_CUDA(c, cudaMemcpyAsync(part.data(), c->red_tmp, 8 * part.size(), cudaMemcpyDeviceToHost, c->stream));
  CUBE_CUDA(c, cudaStreamSynchronize(c->stream));
  r = cube_stats_fetch(c);
  if (r) return r;
  if (c->hstats->flags & 2)
    return cube_fail(c, CUBE_ERR_COUNT_MISMATCH, "a re-sorted particle had no rank in its destination cell");
  double sums[3] = {0, 0, 0};
  for (int b = 0; b < nb; b++)
    for (int t = 0; t < 3; t++) sums[t] += part[3 * b + t];
  c->cur = kn;
  c->np = np_new;
  double npg = (double)(c->npglobal > 0 ? c->npglobal : np_new);
  double std_res = std::sqrt(sums[1] / npg);
  c->sigma_vi_new = (float)(std_res / (double)std::sqrt(3.0f));  // update_particle.f90:224
  if (st) {
    st->nplocal = np_new;
    st->max_tile_np = 0;
    st->nlost = (int64_t)hs.nlost;
    st->ndup = (int64_t)hs.ndup_list;
    st->sum_c = sums[0];
    st->sum_r = sums[1];
    st->sum_s = sums[2];
    st->sigma_vi_new = c->sigma_vi_new;
    st->nlayer = nlayer;
    st->max_disp = hs.max_disp;
    st->rank_walked = c->rank_walked;
  }
  return CUBE_OK;
}
