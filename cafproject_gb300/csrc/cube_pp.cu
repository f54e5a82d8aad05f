// cube_pp.cu -- ext_pp_force (ext_pp_force.f90:10-162) on GB300.
//
// The reference threads a linked list through the fine cells of each tile
// (hoc/ll, ext_pp_force.f90:53-75) and, for every particle of a physical fine
// cell, sums m*r/|r|^3*pcut(|r|) over the particles of the 3^3 neighbouring
// fine cells, skipping pairs with |r| <= rsoft (:94-110), in FP64.  Here the
// particles are already sorted by coarse cell, so a fine neighbourhood is at
// most 2x2x2 coarse cells: a particle in fine sub-cell 0 (3) of its coarse
// cell also reads the coarse cell below (above) in that dimension.  The pair
// arithmetic is FP32 (positions are exact in FP32: 4*frac has <= 17 bits);
// the kick adds F*a_mid*dt/(6 pi) in FP64 (:116) as one product with the
// precomputed factor -- the FP32 pair sum already sets the tolerance of this
// kick, so the reference's two FP64 divisions buy nothing here -- and the
// velocity re-encode is the exact code of update_particle.f90:117.
#include <cmath>

#include "cube_internal.cuh"

namespace {

struct PPArgs {
  Geo g;
  int64_t np;
  const void* xp;
  void* vp;
  const int32_t* pcell;
  const int64_t* cstart;
  CodecView cv;
  float mass, rsoft, inv_cut;
  double kick;   // a_mid*dt/6/pi
  float kick_f;  // the same rounded to float (fast path)
  int exact_only;
  float* fpp;  // optional per-particle force output
  DevStats* st;
};

__device__ __forceinline__ float fine_off(int code, int izipx) {
  // ncell*(int(xp+ishift)+rshift)*x_resolution: exact in real(4)
  return __fmul_rn(pos_off_f(code, izipx), izipx == 1 ? 4.0f / 256.0f : 4.0f / 65536.0f);
}

__global__ void k_pp(PPArgs a) {
  const Geo& g = a.g;
  unsigned long long npairs = 0, nwork = 0;
  float f2max = 0.f;
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < a.np; p += (int64_t)gridDim.x * blockDim.x) {
    int gc[3];
    cell_coords(g, a.pcell[p], gc[0], gc[1], gc[2]);
    float x1[3];
    int fi[3], lo[3], hi[3];
    for (int d = 0; d < 3; d++) {
      x1[d] = fine_off(load_code(a.xp, 3 * p + d, g.izipx), g.izipx);
      fi[d] = (int)floorf(x1[d]);
      lo[d] = fi[d] == 0 ? -1 : 0;
      hi[d] = fi[d] == g.ncell - 1 ? 1 : 0;
    }
    float F[3] = {0.f, 0.f, 0.f};
    for (int dz = lo[2]; dz <= hi[2]; dz++)
      for (int dy = lo[1]; dy <= hi[1]; dy++)
        for (int dx = lo[0]; dx <= hi[0]; dx++) {
          int sx = wrap1(gc[0] + dx, g.nc), sy = wrap1(gc[1] + dy, g.nc), sz = wrap1(gc[2] + dz, g.nc);
          int64_t S = cell_id(g, sx, sy, sz);
          int64_t q0 = a.cstart[S], q1 = a.cstart[S + 1];
          float sh[3] = {(float)(4 * dx), (float)(4 * dy), (float)(4 * dz)};
          for (int64_t q = q0; q < q1; q++) {
            float r[3];
            bool near = true;
            for (int d = 0; d < 3; d++) {
              float x2 = sh[d] + fine_off(load_code(a.xp, 3 * q + d, g.izipx), g.izipx);
              int f2 = (int)floorf(x2);
              near = near && abs(f2 - fi[d]) <= 1;
              r[d] = x2 - x1[d];
            }
            if (!near) continue;
            npairs++;
            float r2 = r[0] * r[0] + r[1] * r[1] + r[2] * r[2];
            float rm = sqrtf(r2);
            if (!(rm > a.rsoft)) continue;  // merge(force,0,rmag>rsoft); self pairs have rm=0
            float rc = rm * a.inv_cut;
            float rc2 = rc * rc;
            float pcut = 1.0f - 1.75f * rc2 * rc + 0.75f * rc2 * rc2 * rc;
            float s = a.mass * pcut / (r2 * rm);
            F[0] += s * r[0];
            F[1] += s * r[1];
            F[2] += s * r[2];
          }
        }
    nwork++;
    for (int d = 0; d < 3; d++) {
      int code = load_code(a.vp, 3 * p + d, g.izipv);
      // vreal=vreal+f_tot*a_mid*dt/6/pi (ext_pp_force.f90:116), then the code:
      // FP32 estimate certified against the FP64 expression (see certify_abs)
      float dh = codec_decode_ff(a.cv, code).x;
      float kf = __fmul_rn(F[d], a.kick_f);
      float vf = __fadd_rn(dh, kf);
      float E = 1.25f * (fabsf(kf) * 1.3e-7f + (2.f * fabsf(dh) + fabsf(vf)) * 6.0e-8f);
      long long n = 0, out;
      if (!a.exact_only && certify_abs(f2d_bits(vf) & 0x7fffffffffffffffLL, E, a.cv, &n)) {
        out = vf < 0.f ? -n : n;
      } else {
        double v = __dadd_rn(codec_decode(a.cv, code), __dmul_rn((double)F[d], a.kick));
        out = codec_encode(a.cv, v);
      }
      store_code(a.vp, 3 * p + d, g.izipv, out);
      if (a.fpp) a.fpp[3 * p + d] = F[d];
    }
    f2max = fmaxf(f2max, F[0] * F[0] + F[1] * F[1] + F[2] * F[2]);
  }
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

}  // namespace

int cube_pp_impl(cube_ctx* c, float a_mid, float dt, cube_stats* st) {
  PPArgs a{};
  int r = cube_codec_pair(c, c->sigma_vi, c->sigma_vi, &a.cv, nullptr);
  if (r) return r;
  CUBE_CUDA(c, cudaMemsetAsync(c->dstats, 0, sizeof(DevStats), c->stream));
  a.g = make_geo(c);
  a.np = c->np;
  a.xp = c->xp[c->cur];
  a.vp = c->vp[c->cur];
  a.pcell = c->pcell[c->cur];
  a.cstart = c->cstart[c->cur];
  a.mass = c->p.mass_p;
  a.rsoft = c->p.rsoft;
  a.inv_cut = 1.0f / (float)c->p.nf_cutoff;
  a.kick = (((double)a_mid * (double)dt) / 6.0) / (double)CUBE_PI_F;
  a.kick_f = (float)a.kick;
  a.exact_only = c->opt_exact_kicks;
  a.fpp = c->fpp;
  a.st = c->dstats;
  cube_phase_begin(c, PH_PP);
  k_pp<<<cube_grid(c->np, 256), 256, 0, c->stream>>>(a);
  cube_phase_end(c, PH_PP);
  CUBE_CUDA(c, cudaGetLastError());
  r = cube_stats_fetch(c);
  if (r) return r;
  if ((int64_t)c->hstats->itest1 != c->np)
    return cube_fail(c, CUBE_ERR_COUNT_MISMATCH, "PP updated a different number of particles than nplocal");
  if (st) {
    st->f2_max_pp = bits_float(c->hstats->f2_pp_bits);
    st->npairs = (int64_t)c->hstats->npairs;
    st->itest1 = (int64_t)c->hstats->itest1;
  }
  return CUBE_OK;
}
