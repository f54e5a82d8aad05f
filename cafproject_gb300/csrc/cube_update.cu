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
  const double* dec;  // decode table for sigma_vi, indexed by v + nvbin/2
  int nvbin;
  double vc;          // vcoef(sigma_vi) for the encode
  int32_t* dest;
  uint8_t* dframe;
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
};

__device__ __forceinline__ double vreal_of(const UpdArgs& a, int64_t p, int d, int64_t cell) {
  int code = load_code(a.vp, 3 * p + d, a.g.izipv);
  return __dadd_rn(a.dec[code + a.nvbin / 2], (double)a.vfield[3 * cell + d]);
}

// global coarse coordinate of tile-local cell l (1-based) of tile coordinate t
__device__ __forceinline__ int glob(const Geo& g, int t, int l) { return wrapi(t * g.nt + l - 1, g.nc); }

// U1: destination of every particle in every frame that sees it.
__global__ void k_dest(UpdArgs a) {
  const Geo& g = a.g;
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  int local_max = 0;
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < a.np; p += stride) {
    int64_t cell = a.pcell[p];
    int gc[3];
    cell_coords(g, cell, gc[0], gc[1], gc[2]);
    // per dim: up to two frames (offset o of the local coordinate) that land
    int nval[3];
    int oval[3][2], igv[3][2];
    bool far = false;
    for (int d = 0; d < 3; d++) {
      int H = gc[d] / g.nt, L = gc[d] - H * g.nt + 1;
      double off = __dmul_rn(pos_off(load_code(a.xp, 3 * p + d, g.izipx), g.izipx), xres_of(g.izipx));
      double v = vreal_of(a, p, d, cell);
      double deltax = __dmul_rn(__dmul_rn((double)a.dt_mid, v), 0.25);  // (dt_mid*vreal)/ncell, ncell=4
      nval[d] = 0;
      for (int f = 0; f < 3; f++) {
        int o = f == 0 ? 0 : (f == 1 ? g.nt : -g.nt);
        int Ls = L + o;
        if (Ls < 1 - g.ncb || Ls > g.nt + g.ncb) continue;  // frame does not see this cell
        double xq = __dadd_rn((double)(Ls - 1), off);
        double s = __dadd_rn(xq, deltax);
        double cs = ceil(s);
        if (cs < (double)(1 - 2 * g.ncb) || cs > (double)(g.nt + 2 * g.ncb)) {
          far = true;
          continue;
        }
        int ig = (int)cs;
        if (ig >= 1 && ig <= g.nt && nval[d] < 2) {
          oval[d][nval[d]] = o;
          igv[d][nval[d]] = ig;
          nval[d]++;
          int disp = abs(ig - Ls);
          local_max = max(local_max, disp);
        }
      }
    }
    if (far) atomicOr(&a.st->flags, 1);
    int ncopy = nval[0] * nval[1] * nval[2];
    if (ncopy == 0) {
      a.dest[p] = -1;
      atomicAdd(&a.st->nlost, 1ull);
      continue;
    }
    for (int k = 0; k < ncopy; k++) {
      int sel[3] = {k % nval[0], (k / nval[0]) % nval[1], k / (nval[0] * nval[1])};
      int dg[3];
      for (int d = 0; d < 3; d++) {
        int H = gc[d] / g.nt;
        // frame tile = H - o/nt (periodic in tiles); destination global coordinate
        int T = wrapi(H - oval[d][sel[d]] / g.nt, g.nnt);
        dg[d] = glob(g, T, igv[d][sel[d]]);
      }
      int32_t D = (int32_t)cell_id(g, dg[0], dg[1], dg[2]);
      int fr = 0;
      for (int d = 2; d >= 0; d--) fr = 3 * fr + (oval[d][sel[d]] / g.nt + 1);
      if (k == 0) {
        a.dest[p] = D;
        a.dframe[p] = (uint8_t)fr;
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

// U2: one thread per destination cell walks the sources in visit order.
__global__ void k_rank(UpdArgs a) {
  const Geo& g = a.g;
  int R = min(a.st->max_disp, 2 * g.ncb);
  int64_t nx = (int64_t)(a.st->ndup_list < (unsigned long long)a.xtra_cap ? a.st->ndup_list : (unsigned long long)a.xtra_cap);
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t D = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; D < a.ncells; D += stride) {
    int dgc[3];
    cell_coords(g, D, dgc[0], dgc[1], dgc[2]);
    int T[3], Dl[3];
    for (int d = 0; d < 3; d++) {
      T[d] = dgc[d] / g.nt;
      Dl[d] = dgc[d] - T[d] * g.nt + 1;
    }
    // source z offsets sorted by (layer, k): layer = (k+ncb-1) mod nlayer
    int dz[2 * 16 + 1];
    int nz = 0;
    for (int o = -R; o <= R; o++) {
      int kl = Dl[2] + o;
      if (kl < 1 - g.ncb || kl > g.nt + g.ncb) continue;
      int lay = (kl + g.ncb - 1) % a.nlayer;
      int pos = nz++;
      while (pos > 0) {
        int ko = Dl[2] + dz[pos - 1];
        int lo = (ko + g.ncb - 1) % a.nlayer;
        if (lo > lay || (lo == lay && ko > kl)) {
          dz[pos] = dz[pos - 1];
          pos--;
        } else {
          break;
        }
      }
      dz[pos] = o;
    }
    float acc[3];
    for (int d = 0; d < 3; d++) acc[d] = __double2float_rn(__dmul_rn((double)a.vfield[3 * D + d], kWeightV));
    uint32_t cnt = 0;
    for (int iz = 0; iz < nz; iz++) {
      int kl = Dl[2] + dz[iz];
      int sz = glob(g, T[2], kl);
      // frame offset (in tiles) at which this destination tile sees the source:
      // local coordinate kl vs the source's own tile-local coordinate
      int fz = (kl - (sz - (sz / g.nt) * g.nt + 1)) / g.nt + 1;
      for (int jl = Dl[1] - R; jl <= Dl[1] + R; jl++) {
        if (jl < 1 - g.ncb || jl > g.nt + g.ncb) continue;
        int sy = glob(g, T[1], jl);
        int fy = (jl - (sy - (sy / g.nt) * g.nt + 1)) / g.nt + 1;
        for (int il = Dl[0] - R; il <= Dl[0] + R; il++) {
          if (il < 1 - g.ncb || il > g.nt + g.ncb) continue;
          int sx = glob(g, T[0], il);
          int fx = (il - (sx - (sx / g.nt) * g.nt + 1)) / g.nt + 1;
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
            for (int d = 0; d < 3; d++) {
              double v = vreal_of(a, p, d, S);
              acc[d] = __double2float_rn(__dadd_rn((double)acc[d], v));
            }
          }
        }
      }
    }
    a.cnt_new[D] = (int32_t)cnt;
    for (int d = 0; d < 3; d++)
      a.vfield_new[3 * D + d] = __double2float_rn(__ddiv_rn((double)acc[d], __dadd_rn((double)cnt, kWeightV)));
  }
}

__device__ __forceinline__ void write_particle(const UpdArgs& a, int64_t p, int32_t D, uint32_t r) {
  const Geo& g = a.g;
  if (D < 0 || (int64_t)D >= a.ncells || r >= (uint32_t)a.cnt_new[D]) {
    atomicOr(&a.st->flags, 2);  // rank not assigned: never write outside the new arrays
    return;
  }
  int64_t idx = a.cstart_new[D] + r;
  int64_t cell = a.pcell[p];
  // nint(dt_mid*vreal/(x_resolution*ncell)): the divisor is a power of two
  double inv = g.izipx == 1 ? 64.0 : 16384.0;
  for (int d = 0; d < 3; d++) {
    double v = vreal_of(a, p, d, cell);
    double P = __dmul_rn((double)a.dt_mid, v);
    long long dx = llround(__dmul_rn(P, inv));
    long long x = load_code(a.xp, 3 * p + d, g.izipx);
    store_code(a.xp_new, 3 * idx + d, g.izipx, x + dx);
    double vrel = __dsub_rn(v, (double)a.vfield_new[3 * (int64_t)D + d]);
    store_code(a.vp_new, 3 * idx + d, g.izipv, v_encode(vrel, a.vc, a.nvbin));
  }
  a.pid_new[idx] = a.pid[p];
  a.pcell_new[idx] = D;
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

// sigma_v sums of the new state (update_particle.f90:172-196): per-block FP64
// partials in a fixed partition, summed in block order on the host.
__global__ void k_sigma(const void* __restrict__ vp, const int32_t* __restrict__ pcell, const float* __restrict__ vfield,
                        int64_t np, int64_t ncells, const double* __restrict__ dec, int nvbin, int izipv,
                        double* __restrict__ part) {
  __shared__ double s[3][32];
  double sc = 0, sr = 0, ss = 0;
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  int64_t t0 = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  for (int64_t c = t0; c < ncells; c += stride) {
    float a0 = vfield[3 * c], a1 = vfield[3 * c + 1], a2 = vfield[3 * c + 2];
    float q = __fadd_rn(__fadd_rn(__fmul_rn(a0, a0), __fmul_rn(a1, a1)), __fmul_rn(a2, a2));
    sc += (double)q;
  }
  for (int64_t p = t0; p < np; p += stride) {
    int64_t c = pcell[p];
    if (c < 0 || c >= ncells) continue;
    double r2 = 0, s2 = 0;
    for (int d = 0; d < 3; d++) {
      double v = dec[load_code(vp, 3 * p + d, izipv) + nvbin / 2];
      r2 += v * v;
      double w = v + (double)vfield[3 * c + d];
      s2 += w * w;
    }
    sr += r2;
    ss += s2;
  }
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

}  // namespace

int cube_update_x_impl(cube_ctx* c, float dt_old, float dt, float vz_max, cube_stats* st) {
  Geo g = make_geo(c);
  int k = c->cur, kn = 1 - k;
  float dt_mid = (dt_old + dt) / 2.0f;  // update_particle.f90:32
  // nlayer=2*ceiling(dt_mid*sim%vz_max/ncell)+1 in real(4) (update_particle.f90:37)
  volatile float q = dt_mid * vz_max;
  volatile float q2 = q / (float)c->p.ncell;
  int nlayer = 2 * (int)std::ceil((double)q2) + 1;
  if (nlayer < 1) nlayer = 1;
  int r = cube_ensure_decode(c, c->dec_old, c->sigma_vi, c->dec_old_sigma);
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
  a.dec = c->dec_old;
  a.nvbin = c->nvbin;
  {
    float s = std::sqrt(CUBE_PI_F / 2.0f);
    a.vc = (double)s / ((double)c->sigma_vi * 2.5);
  }
  a.dest = c->dest;
  a.dframe = c->dframe;
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
  const int B = 256;
  CUBE_CUDA(c, cudaMemsetAsync(c->rank, 0xFF, 4 * (size_t)c->np, c->stream));  // "no rank" sentinel
  cube_phase_begin(c, PH_UPD_DEST);
  k_dest<<<cube_grid(c->np, B), B, 0, c->stream>>>(a);
  cube_phase_end(c, PH_UPD_DEST);
  cube_phase_begin(c, PH_UPD_RANK);
  k_rank<<<cube_grid(c->ncells, 128, 32), 128, 0, c->stream>>>(a);
  cube_phase_end(c, PH_UPD_RANK);
  CUBE_CUDA(c, cudaGetLastError());
  cube_phase_begin(c, PH_UPD_SCAN);
  r = cube_scan_counts(c, c->rhoc[kn], c->cstart[kn], c->ncells);
  cube_phase_end(c, PH_UPD_SCAN);
  if (r) return r;
  int64_t np_new = 0;
  CUBE_CUDA(c, cudaMemcpyAsync(&np_new, c->cstart[kn] + c->ncells, 8, cudaMemcpyDeviceToHost, c->stream));
  r = cube_stats_fetch(c);
  if (r) return r;
  DevStats hs = *c->hstats;
  if (hs.flags & 1) return cube_fail(c, CUBE_ERR_DISPLACEMENT, "a particle left the double-buffer tile");
  if ((int64_t)hs.ndup_list > c->xtra_cap) return cube_fail(c, CUBE_ERR_TILE_OVERFLOW, "extra-copy list overflow");
  if (np_new > c->p.np_max)
    return cube_fail(c, CUBE_ERR_IMAGE_OVERFLOW, "new particle count exceeds np_max");
  cube_phase_begin(c, PH_UPD_SCATTER);
  k_scatter<<<cube_grid(c->np, B), B, 0, c->stream>>>(a);
  if (hs.ndup_list) k_scatter_xtra<<<cube_grid((int64_t)hs.ndup_list, B), B, 0, c->stream>>>(a);
  cube_phase_end(c, PH_UPD_SCATTER);
  CUBE_CUDA(c, cudaGetLastError());
  // sigma statistics of the new state (decoded with sigma_vi)
  int nb = c->red_blocks;
  cube_phase_begin(c, PH_UPD_SIGMA);
  k_sigma<<<nb, 256, 0, c->stream>>>(c->vp[kn], c->pcell[kn], c->vfield[kn], np_new, c->ncells, c->dec_old,
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
  }
  return CUBE_OK;
}
