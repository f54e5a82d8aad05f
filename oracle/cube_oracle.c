/*
 * cube_oracle.c -- CPU restatement of CUBE's per-step drift/re-sort, PM and
 * PP loops (CUBEnu/work/main), used ONLY as test infrastructure: the parity
 * checker for the GPU library and the timed CPU baseline.  Nothing in the
 * product links or calls this file.
 *
 * PARITY UNPINNED: the reference is Coarray Fortran + FFTW3f and no Fortran
 * compiler or FFTW exists where this oracle is built, and the reference ships
 * no golden vectors for this path.  Every loop below follows the cited
 * reference lines statement by statement (loop order, the layered k order,
 * mixed FP32/FP64 promotion, Fortran NINT/CEILING/FLOOR and integer(1/2)
 * wrap-around), and is pinned by the analytic known-answer tests in
 * tests/test_oracle_kat.py.
 *
 * Layout: all arrays use the reference's Fortran (column-major) layouts.
 *   xp(3,np) int8/int16, vp(3,np) int8/int16, pid(np) int32,
 *   rhoc(nt,nt,nt,nnt,nnt,nnt) int32 physical counts,
 *   vfield(3,nt,nt,nt,nnt,nnt,nnt) float.
 * The "buffered state" (variables.f90:44-62 after buffer_grid/buffer_x/
 * buffer_v) is built explicitly by orc_buffer: each tile's extended region
 * 1-ncb..nt+ncb holds periodic copies of the neighbouring cells' particles in
 * their stored order, which is what buffer_grid.f90:124-209 and
 * buffer_particle.f90:27-357 produce on one coarray image.
 *
 * Build: -O2 -ffp-contract=off (no FMA contraction), OpenMP.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* pi=4*atan(1.) in default (single) precision (parameters.f90:67). */
#define PI_F 3.14159274101257324f

typedef struct {
  int64_t nc, nnt, nt, ncell, ncb;
  int64_t izipx, izipv;
  int64_t nf_cutoff, pp_range;
  float rsoft;
  float mass_p;
  int32_t nthreads; /* 1: serial (parity); else OpenMP over k slabs as the reference */
  int32_t tile_sel; /* -1: every tile; t: only tile t (timed CPU sample) */
} orc_params;

/* ---------------------------------------------------------------- helpers */

static inline int32_t ld_i(const void* a, int64_t idx, int64_t nbytes) {
  if (nbytes == 1) return ((const int8_t*)a)[idx];
  return ((const int16_t*)a)[idx];
}
static inline void st_i(void* a, int64_t idx, int64_t nbytes, int64_t v) {
  /* Fortran integer(1/2) assignment of an out-of-range value wraps modulo
     2^(8*nbytes) (gfortran); the C conversion below does the same on gcc. */
  if (nbytes == 1) ((int8_t*)a)[idx] = (int8_t)(uint8_t)(uint64_t)v;
  else ((int16_t*)a)[idx] = (int16_t)(uint16_t)(uint64_t)v;
}
/* int(xp+ishift,izipx)+rshift == unsigned(xp)+0.5: the stored integer wraps
   into the signed izipx-byte range, then shifts back (update_particle.f90:66,
   pm.f90:63; parameters.f90:16-18). */
static inline double off_of(int32_t x, int64_t izipx) {
  int64_t ishift = -((int64_t)1 << (izipx * 8 - 1));
  int64_t m = (int64_t)1 << (izipx * 8);
  int64_t w = (int64_t)x + ishift;
  w = ((w % m) + m) % m;
  if (w >= m / 2) w -= m;
  double rshift = 0.5 - (double)ishift;
  return (double)w + rshift;
}
/* x_resolution=1.0/(2**(izipx*8)) (parameters.f90:119) */
static inline double xres_of(int64_t izipx) { return 1.0 / (double)((int64_t)1 << (8 * izipx)); }
/* ncell*(i-1)+ncell*(int(xp+ishift)+rshift)*x_resolution in real(8)
   (pm.f90:63, ext_pp_force.f90:66) */
static inline double fine_pos(int64_t ncell, int64_t cell, int32_t x, int64_t izipx) {
  return (double)(ncell * (cell - 1)) + ((double)ncell * off_of(x, izipx)) * xres_of(izipx);
}
/* (cell-1)+(int(xp+ishift)+rshift)*x_resolution-0.5 (pm.f90:221,335) */
static inline double coarse_pos(int64_t cell, int32_t x, int64_t izipx) {
  return ((double)(cell - 1) + off_of(x, izipx) * xres_of(izipx)) - 0.5;
}
/* Fortran NINT: nearest integer, halves away from zero. */
static inline int64_t f_nint(double x) { return (int64_t)llround(x); }
/* Fortran CEILING / FLOOR of a real(8) returning integer(8). */
static inline int64_t f_ceil(double x) { return (int64_t)ceil(x); }

/* sqrt(pi/2)/(sigma*vrel_boost): real(4) sqrt over a real(8) product
   (update_particle.f90:67, variables.f90:36, parameters.f90:123). */
static inline double vcoef(float sigma) {
  float s = sqrtf(PI_F / 2.0f);
  return (double)s / ((double)sigma * 2.5);
}
/* vreal = tan(pi*real(vp)/real(nvbin-1)) / vcoef  (update_particle.f90:67).
   The FP32 tan is taken as the correctly rounded value float(tan(double)). */
static inline double v_decode(int32_t v, double c, int64_t izipv) {
  float nvm1 = (float)(((int64_t)1 << (8 * izipv)) - 1);
  float arg = (PI_F * (float)v) / nvm1;
  float t = (float)tan((double)arg);
  return (double)t / c;
}
/* vp = nint(real(nvbin-1)*atan(vcoef*vreal)/pi, kind=izipv)
   (update_particle.f90:117, pm.f90:158). */
static inline int64_t v_encode(double v, double c, int64_t izipv) {
  float nvm1 = (float)(((int64_t)1 << (8 * izipv)) - 1);
  double u = ((double)nvm1 * atan(c * v)) / (double)PI_F;
  return f_nint(u);
}

/* extended-cell linear index, local cell (i,j,k) in [1-ncb, nt+ncb] */
static inline int64_t ext_index(const orc_params* p, int64_t i, int64_t j, int64_t k, int64_t t) {
  int64_t nte = p->nt + 2 * p->ncb;
  return (i + p->ncb - 1) + nte * ((j + p->ncb - 1) + nte * ((k + p->ncb - 1) + nte * t));
}
/* physical cell id in the disjoint (checkpoint) order, global 0-based coords */
static inline int64_t phys_index(const orc_params* p, int64_t gx, int64_t gy, int64_t gz) {
  int64_t nt = p->nt, nnt = p->nnt;
  int64_t tx = gx / nt, ty = gy / nt, tz = gz / nt;
  int64_t ix = gx % nt, iy = gy % nt, iz = gz % nt;
  return ix + nt * (iy + nt * (iz + nt * (tx + nnt * (ty + nnt * tz))));
}
static inline int64_t wrapc(int64_t g, int64_t n) { return ((g % n) + n) % n; }

static void set_threads(const orc_params* p) {
#ifdef _OPENMP
  if (p->nthreads > 0) omp_set_num_threads(p->nthreads);
#else
  (void)p;
#endif
}

/* ------------------------------------------------------- buffered state */

/* Number of particle slots of the buffered state (sum of extended counts). */
int64_t orc_buffer_count(const orc_params* p, const int32_t* rhoc) {
  int64_t nt = p->nt, nnt = p->nnt, ncb = p->ncb, nc = p->nc, tot = 0;
  for (int64_t t = 0; t < nnt * nnt * nnt; t++) {
    int64_t tx = t % nnt, ty = (t / nnt) % nnt, tz = t / (nnt * nnt);
    for (int64_t k = 1 - ncb; k <= nt + ncb; k++)
      for (int64_t j = 1 - ncb; j <= nt + ncb; j++)
        for (int64_t i = 1 - ncb; i <= nt + ncb; i++) {
          int64_t gx = wrapc(tx * nt + i - 1, nc), gy = wrapc(ty * nt + j - 1, nc),
                  gz = wrapc(tz * nt + k - 1, nc);
          tot += rhoc[phys_index(p, gx, gy, gz)];
        }
  }
  return tot;
}

/* Build the buffered state from the disjoint state: brhoc/bvfield are the
   periodic extension of rhoc/vfield (buffer_np/buffer_vc,
   buffer_grid.f90:28-122); bstart is the exclusive spine over extended cells
   (nzero of update_particle.f90:63 == idx_b_r - sum(rhoc(i:,j,k)),
   spine_image variables.f90:141-187); bxp/bvp/bpid hold each extended cell's
   particles copied in stored order (redistribute_cdm + buffer_xvp).  The
   spine is one serial prefix sum over the extended cells; the copies run in
   parallel over them. */
void orc_buffer(const orc_params* p, const void* xp, const void* vp, const int32_t* pid,
                const int32_t* rhoc, const float* vfield, int32_t* brhoc, float* bvfield,
                int64_t* bstart, void* bxp, void* bvp, int32_t* bpid) {
  int64_t nt = p->nt, nnt = p->nnt, ncb = p->ncb, nc = p->nc, nte = nt + 2 * ncb;
  int64_t ncell_phys = nc * nc * nc, next = nte * nte * nte * nnt * nnt * nnt;
  int64_t* cstart = (int64_t*)malloc(sizeof(int64_t) * (ncell_phys + 1));
  int64_t* src_of = (int64_t*)malloc(sizeof(int64_t) * next);
  cstart[0] = 0;
  for (int64_t c = 0; c < ncell_phys; c++) cstart[c + 1] = cstart[c] + rhoc[c];
  set_threads(p);
  /* the physical cell behind every extended cell, its count and field */
#pragma omp parallel for schedule(static)
  for (int64_t e = 0; e < next; e++) {
    int64_t i = e % nte, j = (e / nte) % nte, k = (e / (nte * nte)) % nte, t = e / (nte * nte * nte);
    int64_t tx = t % nnt, ty = (t / nnt) % nnt, tz = t / (nnt * nnt);
    int64_t gx = wrapc(tx * nt + i - ncb, nc), gy = wrapc(ty * nt + j - ncb, nc), gz = wrapc(tz * nt + k - ncb, nc);
    int64_t c = phys_index(p, gx, gy, gz);
    src_of[e] = c;
    brhoc[e] = rhoc[c];
    for (int d = 0; d < 3; d++) bvfield[3 * e + d] = vfield[3 * c + d];
  }
  int64_t pos = 0;
  for (int64_t e = 0; e < next; e++) {
    bstart[e] = pos;
    pos += brhoc[e];
  }
#pragma omp parallel for schedule(dynamic, 4096)
  for (int64_t e = 0; e < next; e++) {
    int64_t c = src_of[e];
    for (int64_t l = 0; l < brhoc[e]; l++) {
      int64_t src = cstart[c] + l, dst = bstart[e] + l;
      for (int d = 0; d < 3; d++) {
        st_i(bxp, 3 * dst + d, p->izipx, ld_i(xp, 3 * src + d, p->izipx));
        st_i(bvp, 3 * dst + d, p->izipv, ld_i(vp, 3 * src + d, p->izipv));
      }
      if (pid && bpid) bpid[dst] = pid[src];
    }
  }
  free(src_of);
  free(cstart);
}

/* Copy the physical cells of the buffered state back to the disjoint layout
   (the particle order of checkpoint.f90:38-47), in parallel over cells. */
void orc_unbuffer(const orc_params* p, const int32_t* brhoc, const int64_t* bstart, const void* bxp,
                  const void* bvp, const int32_t* bpid, void* xp, void* vp, int32_t* pid) {
  int64_t nt = p->nt, nnt = p->nnt, ncell = nt * nt * nt * nnt * nnt * nnt;
  int64_t* out = (int64_t*)malloc(sizeof(int64_t) * (ncell + 1));
  out[0] = 0;
  /* physical cells in the disjoint order: tile, then k, j, i inside it */
  for (int64_t c = 0; c < ncell; c++) {
    int64_t i = c % nt + 1, j = (c / nt) % nt + 1, k = (c / (nt * nt)) % nt + 1, t = c / (nt * nt * nt);
    out[c + 1] = out[c] + brhoc[ext_index(p, i, j, k, t)];
  }
  set_threads(p);
#pragma omp parallel for schedule(dynamic, 4096)
  for (int64_t c = 0; c < ncell; c++) {
    int64_t i = c % nt + 1, j = (c / nt) % nt + 1, k = (c / (nt * nt)) % nt + 1, t = c / (nt * nt * nt);
    int64_t e = ext_index(p, i, j, k, t);
    for (int64_t l = 0; l < brhoc[e]; l++) {
      int64_t src = bstart[e] + l, dst = out[c] + l;
      for (int d = 0; d < 3; d++) {
        st_i(xp, 3 * dst + d, p->izipx, ld_i(bxp, 3 * src + d, p->izipx));
        st_i(vp, 3 * dst + d, p->izipv, ld_i(bvp, 3 * src + d, p->izipv));
      }
      if (pid && bpid) pid[dst] = bpid[src];
    }
  }
  free(out);
}

/* ------------------------------------------------------------- update_xp */

/* Drift + counting re-sort of one image, update_xp (update_particle.f90:16-167).
   Inputs are the buffered state; outputs the new disjoint state.
   flags bit0: a destination cell fell outside the double-buffer tile
   (the reference would index rhoce out of bounds). Returns nplocal. */
int64_t orc_update_xp(const orc_params* p, float dt_mid, float vz_max, float sigma_vi,
                      const int32_t* brhoc, const int64_t* bstart, const float* bvfield,
                      const void* bxp, const void* bvp, const int32_t* bpid, void* xp_out,
                      void* vp_out, int32_t* pid_out, int32_t* rhoc_out, float* vfield_out,
                      int64_t* max_tile_np, int32_t* flags) {
  int64_t nt = p->nt, nnt = p->nnt, ncb = p->ncb, ncell = p->ncell;
  int64_t ne2 = nt + 4 * ncb; /* double-buffer tile 1-2ncb..nt+2ncb */
  int64_t ne2c = ne2 * ne2 * ne2;
  const double weight_v = (double)0.1f; /* real(8),parameter :: weight_v=0.1 (a real(4) literal) */
  const double xres = xres_of(p->izipx);
  const double c = vcoef(sigma_vi);
  /* nlayer=2*ceiling(dt_mid*sim%vz_max/ncell)+1 in real(4) (update_particle.f90:37) */
  float q = (dt_mid * vz_max) / (float)ncell;
  int64_t nlayer = 2 * (int64_t)ceilf(q) + 1;
  int32_t* rhoce = (int32_t*)malloc(sizeof(int32_t) * ne2c);
  int32_t* rholocal = (int32_t*)malloc(sizeof(int32_t) * ne2c);
  float* vnew = (float*)malloc(sizeof(float) * 3 * ne2c);
  int64_t* estart = (int64_t*)malloc(sizeof(int64_t) * (ne2c + 1));
  int64_t cap = 0;
  for (int64_t t = 0; t < nnt * nnt * nnt; t++) {
    int64_t s = 0;
    for (int64_t k = 1 - ncb; k <= nt + ncb; k++)
      for (int64_t j = 1 - ncb; j <= nt + ncb; j++)
        for (int64_t i = 1 - ncb; i <= nt + ncb; i++) s += brhoc[ext_index(p, i, j, k, t)];
    if (s > cap) cap = s;
  }
  int64_t psz = p->izipx > p->izipv ? p->izipx : p->izipv;
  void* xnew = malloc((size_t)(3 * cap * psz + 16));
  void* vnewp = malloc((size_t)(3 * cap * psz + 16));
  int32_t* pnew = (int32_t*)malloc(sizeof(int32_t) * (cap + 1));
  int64_t np_prev = 0, maxnp = 0;
  int par = p->nthreads != 1;
  set_threads(p);
#define E2(i, j, k) (((i) + 2 * ncb - 1) + ne2 * (((j) + 2 * ncb - 1) + ne2 * ((k) + 2 * ncb - 1)))
  for (int64_t t = 0; t < nnt * nnt * nnt; t++) {
    if (p->tile_sel >= 0 && t != p->tile_sel) continue;
    memset(rhoce, 0, sizeof(int32_t) * ne2c);
    memset(rholocal, 0, sizeof(int32_t) * ne2c);
    memset(vnew, 0, sizeof(float) * 3 * ne2c);
    /* vfield_new(:,1-ncb:nt+ncb,...)=vfield*weight_v (update_particle.f90:47-48) */
    for (int64_t k = 1 - ncb; k <= nt + ncb; k++)
      for (int64_t j = 1 - ncb; j <= nt + ncb; j++)
        for (int64_t i = 1 - ncb; i <= nt + ncb; i++) {
          int64_t e = ext_index(p, i, j, k, t);
          for (int d = 0; d < 3; d++) vnew[3 * E2(i, j, k) + d] = (float)((double)bvfield[3 * e + d] * weight_v);
        }
    /* pass 1: density + vfield (update_particle.f90:55-78), layered k order;
       slabs of one layer run in parallel as the reference's OpenMP loop */
    int32_t fl = 0;
    for (int64_t ilayer = 0; ilayer < nlayer; ilayer++) {
      int64_t nk = (nt + ncb - (1 - ncb + ilayer)) / nlayer + 1;
#pragma omp parallel for schedule(static, 2) if (par) reduction(| : fl)
      for (int64_t kk = 0; kk < nk; kk++) {
        int64_t k = 1 - ncb + ilayer + kk * nlayer;
        for (int64_t j = 1 - ncb; j <= nt + ncb; j++)
          for (int64_t i = 1 - ncb; i <= nt + ncb; i++) {
            int64_t e = ext_index(p, i, j, k, t);
            int64_t cidx[3] = {i, j, k};
            for (int64_t l = 0; l < brhoc[e]; l++) {
              int64_t ip = bstart[e] + l;
              int64_t ig[3];
              double vr[3];
              for (int d = 0; d < 3; d++) {
                double xq = ((double)cidx[d] - 1.0) + off_of(ld_i(bxp, 3 * ip + d, p->izipx), p->izipx) * xres;
                vr[d] = v_decode(ld_i(bvp, 3 * ip + d, p->izipv), c, p->izipv) + (double)bvfield[3 * e + d];
                double deltax = ((double)dt_mid * vr[d]) / (double)ncell;
                ig[d] = f_ceil(xq + deltax);
              }
              if (ig[0] < 1 - 2 * ncb || ig[0] > nt + 2 * ncb || ig[1] < 1 - 2 * ncb || ig[1] > nt + 2 * ncb ||
                  ig[2] < 1 - 2 * ncb || ig[2] > nt + 2 * ncb) {
                fl |= 1;
                continue;
              }
              int64_t g = E2(ig[0], ig[1], ig[2]);
              rhoce[g]++;
              for (int d = 0; d < 3; d++) vnew[3 * g + d] = (float)((double)vnew[3 * g + d] + vr[d]);
            }
          }
      }
    }
    *flags |= fl;
    /* vfield_new=vfield_new/(rhoce+weight_v) (update_particle.f90:81-83) */
    for (int64_t g = 0; g < ne2c; g++)
      for (int d = 0; d < 3; d++) vnew[3 * g + d] = (float)((double)vnew[3 * g + d] / ((double)rhoce[g] + weight_v));
    /* spine_tile (variables.f90:96-139): start of each double-buffer cell */
    estart[0] = 0;
    for (int64_t g = 0; g < ne2c; g++) estart[g + 1] = estart[g] + rhoce[g];
    if (estart[ne2c] > maxnp) maxnp = estart[ne2c];
    /* pass 2: scatter (update_particle.f90:97-126) */
    for (int64_t ilayer = 0; ilayer < nlayer; ilayer++) {
      int64_t nk = (nt + ncb - (1 - ncb + ilayer)) / nlayer + 1;
#pragma omp parallel for schedule(static, 2) if (par)
      for (int64_t kk = 0; kk < nk; kk++) {
        int64_t k = 1 - ncb + ilayer + kk * nlayer;
        for (int64_t j = 1 - ncb; j <= nt + ncb; j++)
          for (int64_t i = 1 - ncb; i <= nt + ncb; i++) {
            int64_t e = ext_index(p, i, j, k, t);
            int64_t cidx[3] = {i, j, k};
            for (int64_t l = 0; l < brhoc[e]; l++) {
              int64_t ip = bstart[e] + l;
              int64_t ig[3];
              double vr[3];
              for (int d = 0; d < 3; d++) {
                double xq = ((double)cidx[d] - 1.0) + off_of(ld_i(bxp, 3 * ip + d, p->izipx), p->izipx) * xres;
                vr[d] = v_decode(ld_i(bvp, 3 * ip + d, p->izipv), c, p->izipv) + (double)bvfield[3 * e + d];
                double deltax = ((double)dt_mid * vr[d]) / (double)ncell;
                ig[d] = f_ceil(xq + deltax);
              }
              if (ig[0] < 1 - 2 * ncb || ig[0] > nt + 2 * ncb || ig[1] < 1 - 2 * ncb || ig[1] > nt + 2 * ncb ||
                  ig[2] < 1 - 2 * ncb || ig[2] > nt + 2 * ncb)
                continue;
              int64_t g = E2(ig[0], ig[1], ig[2]);
              rholocal[g]++;
              int64_t idx = estart[g] + rholocal[g] - 1;
              for (int d = 0; d < 3; d++) {
                int64_t dx = f_nint(((double)dt_mid * vr[d]) / (xres * (double)ncell));
                st_i(xnew, 3 * idx + d, p->izipx, (int64_t)ld_i(bxp, 3 * ip + d, p->izipx) + dx);
                double vrel = vr[d] - (double)vnew[3 * g + d];
                st_i(vnewp, 3 * idx + d, p->izipv, v_encode(vrel, c, p->izipv));
              }
              pnew[idx] = bpid ? bpid[ip] : 0;
            }
          }
      }
    }
    /* delete buffer particles, write rhoc/vfield (update_particle.f90:132-147) */
    int64_t tbase = t * nt * nt * nt;
    for (int64_t k = 1; k <= nt; k++)
      for (int64_t j = 1; j <= nt; j++)
        for (int64_t i = 1; i <= nt; i++) {
          int64_t g = E2(i, j, k);
          int64_t cphys = tbase + (i - 1) + nt * ((j - 1) + nt * (k - 1));
          rhoc_out[cphys] = rhoce[g];
          for (int d = 0; d < 3; d++) vfield_out[3 * cphys + d] = vnew[3 * g + d];
          for (int64_t l = 0; l < rhoce[g]; l++) {
            int64_t src = estart[g] + l;
            for (int d = 0; d < 3; d++) {
              st_i(xp_out, 3 * np_prev + d, p->izipx, ld_i(xnew, 3 * src + d, p->izipx));
              st_i(vp_out, 3 * np_prev + d, p->izipv, ld_i(vnewp, 3 * src + d, p->izipv));
            }
            if (pid_out) pid_out[np_prev] = pnew[src];
            np_prev++;
          }
        }
  }
#undef E2
  if (max_tile_np) *max_tile_np = maxnp;
  free(rhoce);
  free(rholocal);
  free(vnew);
  free(estart);
  free(xnew);
  free(vnewp);
  free(pnew);
  return np_prev;
}

/* sigma_v statistics of a disjoint state (update_particle.f90:172-224):
   out[0]=sum_c, out[1]=sum_r, out[2]=sum_s (FP64 sums, serial order). */
void orc_sigma_sums(const orc_params* p, float sigma_vi, const void* vp, const int32_t* rhoc,
                    const float* vfield, double* out) {
  int64_t ncells = p->nc * p->nc * p->nc, ip = 0;
  double c = vcoef(sigma_vi), sc = 0, sr = 0, ss = 0;
  for (int64_t cl = 0; cl < ncells; cl++) {
    float vc2 = vfield[3 * cl] * vfield[3 * cl];
    vc2 = vc2 + vfield[3 * cl + 1] * vfield[3 * cl + 1];
    vc2 = vc2 + vfield[3 * cl + 2] * vfield[3 * cl + 2];
    sc = sc + (double)vc2;
    for (int64_t l = 0; l < rhoc[cl]; l++, ip++) {
      double vr[3];
      for (int d = 0; d < 3; d++) vr[d] = v_decode(ld_i(vp, 3 * ip + d, p->izipv), c, p->izipv);
      sr = sr + ((vr[0] * vr[0] + vr[1] * vr[1]) + vr[2] * vr[2]);
      for (int d = 0; d < 3; d++) vr[d] = vr[d] + (double)vfield[3 * cl + d];
      ss = ss + ((vr[0] * vr[0] + vr[1] * vr[1]) + vr[2] * vr[2]);
    }
  }
  out[0] = sc;
  out[1] = sr;
  out[2] = ss;
}

/* ------------------------------------------------------------- fine PM */

/* CIC of one particle at fine position cidx (tile-local coarse cell, 1-based)
   into rho(nfe,nfe,nfe) with the reference's real(4) weights (pm.f90:62-78). */
static inline void fine_cic(int64_t ncell, int64_t nfb, int64_t nfe, const int64_t cidx[3], const void* bxp,
                            int64_t ip, int64_t izipx, float mass, float* rho) {
  int64_t i1[3], i2[3];
  float d1[3], d2[3];
  for (int d = 0; d < 3; d++) {
    double tx = fine_pos(ncell, cidx[d], ld_i(bxp, 3 * ip + d, izipx), izipx);
    float tempx = (float)tx;
    i1[d] = (int64_t)floorf(tempx) + 1;
    i2[d] = i1[d] + 1;
    d1[d] = (float)i1[d] - tempx;
    d2[d] = 1.0f - d1[d];
    i1[d] += nfb;
    i2[d] += nfb;
  }
#define RF(a, b, c) rho[((a)-1) + nfe * (((b)-1) + nfe * ((c)-1))]
  RF(i1[0], i1[1], i1[2]) += ((d1[0] * d1[1]) * d1[2]) * mass;
  RF(i2[0], i1[1], i1[2]) += ((d2[0] * d1[1]) * d1[2]) * mass;
  RF(i1[0], i2[1], i1[2]) += ((d1[0] * d2[1]) * d1[2]) * mass;
  RF(i1[0], i1[1], i2[2]) += ((d1[0] * d1[1]) * d2[2]) * mass;
  RF(i1[0], i2[1], i2[2]) += ((d1[0] * d2[1]) * d2[2]) * mass;
  RF(i2[0], i1[1], i2[2]) += ((d2[0] * d1[1]) * d2[2]) * mass;
  RF(i2[0], i2[1], i1[2]) += ((d2[0] * d2[1]) * d1[2]) * mass;
  RF(i2[0], i2[1], i2[2]) += ((d2[0] * d2[1]) * d2[2]) * mass;
#undef RF
}

/* Fine CIC deposit of tile t into rho(nfe,nfe,nfe) (pm.f90:50-107); rho is
   zeroed here. OpenMP over k slabs 3 apart, as the reference layers them.
   q (may be NULL) is a second species (CUBEnu's neutrinos) with its own
   buffered state: each cell's particles of the second species follow the
   cell's first-species particles into the same mesh (pm.f90:79-103). */
void orc_fine_deposit(const orc_params* p, int64_t t, const int32_t* brhoc, const int64_t* bstart,
                      const void* bxp, float* rho, const orc_params* q, const int32_t* brhoc2,
                      const int64_t* bstart2, const void* bxp2) {
  int64_t nt = p->nt, ncb = p->ncb, ncell = p->ncell;
  int64_t nfb = ncb * ncell, nft = nt * ncell, nfe = nft + 2 * nfb;
  const int64_t nlayer = 3;
  memset(rho, 0, sizeof(float) * nfe * nfe * nfe);
  set_threads(p);
  for (int64_t ilayer = 0; ilayer < nlayer; ilayer++) {
#pragma omp parallel for schedule(static, 2)
    for (int64_t k = 2 - ncb + ilayer; k <= nt + ncb - 1; k += nlayer)
      for (int64_t j = 2 - ncb; j <= nt + ncb - 1; j++)
        for (int64_t i = 2 - ncb; i <= nt + ncb - 1; i++) {
          int64_t e = ext_index(p, i, j, k, t);
          int64_t cidx[3] = {i, j, k};
          for (int64_t l = 0; l < brhoc[e]; l++)
            fine_cic(ncell, nfb, nfe, cidx, bxp, bstart[e] + l, p->izipx, p->mass_p, rho);
          if (q)
            for (int64_t l = 0; l < brhoc2[e]; l++)
              fine_cic(ncell, nfb, nfe, cidx, bxp2, bstart2[e] + l, q->izipx, q->mass_p, rho);
        }
  }
}

/* One CIC-interpolated kick term, evaluated left to right in real(4):
   force*a_mid*dt/6/pi*dxa*dxb*dxc (pm.f90:146-153). */
static inline float kick_term(float f, float a_mid, float dt, float wa, float wb, float wc) {
  float r = f * a_mid;
  r = r * dt;
  r = r / 6.0f;
  r = r / PI_F;
  r = r * wa;
  r = r * wb;
  r = r * wc;
  return r;
}

/* Fine kick of tile t (pm.f90:129-189). force holds force_f(3,nfb:nfe-nfb+1)^3
   as (3,m,m,m) with m=nft+2. Updates bvp of physical particles in place. */
void orc_fine_kick(const orc_params* p, int64_t t, float a_mid, float dt, float sigma_vi,
                   float sigma_vi_new, const int32_t* brhoc, const int64_t* bstart, const void* bxp,
                   void* bvp, const float* force) {
  int64_t nt = p->nt, ncell = p->ncell;
  int64_t nft = nt * ncell, m = nft + 2;
  double c_old = vcoef(sigma_vi), c_new = vcoef(sigma_vi_new);
  set_threads(p);
#pragma omp parallel for schedule(static, 2)
  for (int64_t k = 1; k <= nt; k++)
    for (int64_t j = 1; j <= nt; j++)
      for (int64_t i = 1; i <= nt; i++) {
        int64_t e = ext_index(p, i, j, k, t);
        int64_t cidx[3] = {i, j, k};
        for (int64_t l = 0; l < brhoc[e]; l++) {
          int64_t ip = bstart[e] + l;
          int64_t i1[3], i2[3];
          float d1[3], d2[3];
          for (int d = 0; d < 3; d++) {
            double tx = fine_pos(ncell, cidx[d], ld_i(bxp, 3 * ip + d, p->izipx), p->izipx);
            float tempx = (float)tx;
            i1[d] = (int64_t)floorf(tempx) + 1;
            i2[d] = i1[d] + 1;
            d1[d] = (float)i1[d] - tempx;
            d2[d] = 1.0f - d1[d];
            /* idx+nfb indexes force_f(nfb:nfe-nfb+1); the (3,m,m,m) box is 1-based */
            i1[d] = i1[d] + 1;
            i2[d] = i2[d] + 1;
          }
#define FF(d, a, b, cc) force[(d) + 3 * (((a)-1) + m * (((b)-1) + m * ((cc)-1)))]
          for (int d = 0; d < 3; d++) {
            double vr = v_decode(ld_i(bvp, 3 * ip + d, p->izipv), c_old, p->izipv);
            vr = vr + (double)kick_term(FF(d, i1[0], i1[1], i1[2]), a_mid, dt, d1[0], d1[1], d1[2]);
            vr = vr + (double)kick_term(FF(d, i2[0], i1[1], i1[2]), a_mid, dt, d2[0], d1[1], d1[2]);
            vr = vr + (double)kick_term(FF(d, i1[0], i2[1], i1[2]), a_mid, dt, d1[0], d2[1], d1[2]);
            vr = vr + (double)kick_term(FF(d, i1[0], i1[1], i2[2]), a_mid, dt, d1[0], d1[1], d2[2]);
            vr = vr + (double)kick_term(FF(d, i1[0], i2[1], i2[2]), a_mid, dt, d1[0], d2[1], d2[2]);
            vr = vr + (double)kick_term(FF(d, i2[0], i1[1], i2[2]), a_mid, dt, d2[0], d1[1], d2[2]);
            vr = vr + (double)kick_term(FF(d, i2[0], i2[1], i1[2]), a_mid, dt, d2[0], d2[1], d1[2]);
            vr = vr + (double)kick_term(FF(d, i2[0], i2[1], i2[2]), a_mid, dt, d2[0], d2[1], d2[2]);
            st_i(bvp, 3 * ip + d, p->izipv, v_encode(vr, c_new, p->izipv));
          }
#undef FF
        }
      }
}

/* ----------------------------------------------------------- coarse PM */

/* CIC of one particle into r3t(-1:nt+2)^3 at the coarse position of
   tile-local cell cidx, -0.5 shift (pm.f90:219-233). */
static inline void coarse_cic(int64_t n4, const int64_t cidx[3], const void* bxp, int64_t ip, int64_t izipx,
                              float mass, float* r3t) {
  int64_t i1[3], i2[3];
  float d1[3], d2[3];
  for (int d = 0; d < 3; d++) {
    double tx2 = coarse_pos(cidx[d], ld_i(bxp, 3 * ip + d, izipx), izipx);
    float tempx = (float)tx2;
    i1[d] = (int64_t)floorf(tempx) + 1;
    i2[d] = i1[d] + 1;
    d1[d] = (float)i1[d] - tempx;
    d2[d] = 1.0f - d1[d];
  }
#define RT(a, b, c) r3t[((a) + 1) + n4 * (((b) + 1) + n4 * ((c) + 1))]
  RT(i1[0], i1[1], i1[2]) += ((d1[0] * d1[1]) * d1[2]) * mass;
  RT(i2[0], i1[1], i1[2]) += ((d2[0] * d1[1]) * d1[2]) * mass;
  RT(i1[0], i2[1], i1[2]) += ((d1[0] * d2[1]) * d1[2]) * mass;
  RT(i1[0], i1[1], i2[2]) += ((d1[0] * d1[1]) * d2[2]) * mass;
  RT(i1[0], i2[1], i2[2]) += ((d1[0] * d2[1]) * d2[2]) * mass;
  RT(i2[0], i1[1], i2[2]) += ((d2[0] * d1[1]) * d2[2]) * mass;
  RT(i2[0], i2[1], i1[2]) += ((d2[0] * d2[1]) * d1[2]) * mass;
  RT(i2[0], i2[1], i2[2]) += ((d2[0] * d2[1]) * d2[2]) * mass;
#undef RT
}

/* Coarse CIC deposit of the whole image into r3(nc,nc,nc) (pm.f90:205-267);
   q (may be NULL) is a second species deposited after each cell's
   first-species particles (pm.f90:234-250). */
void orc_coarse_deposit(const orc_params* p, const int32_t* brhoc, const int64_t* bstart,
                        const void* bxp, float* r3, const orc_params* q, const int32_t* brhoc2,
                        const int64_t* bstart2, const void* bxp2) {
  int64_t nt = p->nt, nnt = p->nnt, nc = p->nc;
  int64_t n4 = nt + 4; /* r3t(-1:nt+2)^3 */
  float* r3t = (float*)malloc(sizeof(float) * n4 * n4 * n4);
  memset(r3, 0, sizeof(float) * nc * nc * nc);
  set_threads(p);
  for (int64_t t = 0; t < nnt * nnt * nnt; t++) {
    int64_t tx = t % nnt, ty = (t / nnt) % nnt, tz = t / (nnt * nnt);
    memset(r3t, 0, sizeof(float) * n4 * n4 * n4);
    for (int64_t ilayer = 0; ilayer < 3; ilayer++) {
#pragma omp parallel for schedule(static, 2)
      for (int64_t k = 0 + ilayer; k <= nt + 1; k += 3)
        for (int64_t j = 0; j <= nt + 1; j++)
          for (int64_t i = 0; i <= nt + 1; i++) {
            int64_t e = ext_index(p, i, j, k, t);
            int64_t cidx[3] = {i, j, k};
            for (int64_t l = 0; l < brhoc[e]; l++) coarse_cic(n4, cidx, bxp, bstart[e] + l, p->izipx, p->mass_p, r3t);
            if (q)
              for (int64_t l = 0; l < brhoc2[e]; l++)
                coarse_cic(n4, cidx, bxp2, bstart2[e] + l, q->izipx, q->mass_p, r3t);
          }
    }
#define RT(a, b, c) r3t[((a) + 1) + n4 * (((b) + 1) + n4 * ((c) + 1))]
    for (int64_t k = 1; k <= nt; k++)
      for (int64_t j = 1; j <= nt; j++)
        for (int64_t i = 1; i <= nt; i++)
          r3[(tx * nt + i - 1) + nc * ((ty * nt + j - 1) + nc * (tz * nt + k - 1))] = RT(i, j, k);
#undef RT
  }
  free(r3t);
}

/* Coarse kick (pm.f90:322-387). force_c is (3,nc,nc,nc); the halo
   force_c(:,0,:,:)=force_c(:,nc,:,:) etc. (pm.f90:305-313) is applied as a
   periodic wrap. vmax_out[3] receives max|vreal+vfield| per component;
   vmax_signed (may be NULL) the neutrino loop's statistic
   max(maxval(vreal+vfield_nu)), signed, over the components (pm.f90:377). */
void orc_coarse_kick(const orc_params* p, float a_mid, float dt, float sigma_vi, const int32_t* brhoc,
                     const int64_t* bstart, const float* bvfield, const void* bxp, void* bvp,
                     const float* force_c, float* vmax_out, double* vmax_signed) {
  int64_t nt = p->nt, nnt = p->nnt, nc = p->nc;
  double c = vcoef(sigma_vi);
  double vm[3] = {0, 0, 0};
  double vs = 0; /* vmax_nu starts at 0 (pm.f90:39) */
  set_threads(p);
  for (int64_t t = 0; t < nnt * nnt * nnt; t++) {
    int64_t tl[3] = {t % nnt, (t / nnt) % nnt, t / (nnt * nnt)};
    double v0 = 0, v1 = 0, v2 = 0, vsg = vs;
#pragma omp parallel for schedule(static, 2) reduction(max : v0, v1, v2, vsg)
    for (int64_t k = 1; k <= nt; k++)
      for (int64_t j = 1; j <= nt; j++)
        for (int64_t i = 1; i <= nt; i++) {
          int64_t e = ext_index(p, i, j, k, t);
          int64_t cidx[3] = {i, j, k};
          for (int64_t l = 0; l < brhoc[e]; l++) {
            int64_t ip = bstart[e] + l;
            int64_t i1[3], i2[3];
            float d1[3], d2[3];
            for (int d = 0; d < 3; d++) {
              double tx2 = coarse_pos(tl[d] * nt + cidx[d], ld_i(bxp, 3 * ip + d, p->izipx), p->izipx);
              float tempx = (float)tx2;
              i1[d] = (int64_t)floorf(tempx) + 1;
              i2[d] = i1[d] + 1;
              d1[d] = (float)i1[d] - tempx;
              d2[d] = 1.0f - d1[d];
              i1[d] = wrapc(i1[d] - 1, nc);
              i2[d] = wrapc(i2[d] - 1, nc);
            }
#define FC(d, a, b, cc) force_c[(d) + 3 * ((a) + nc * ((b) + nc * (cc)))]
            for (int d = 0; d < 3; d++) {
              double vr = v_decode(ld_i(bvp, 3 * ip + d, p->izipv), c, p->izipv);
              vr = vr + (double)kick_term(FC(d, i1[0], i1[1], i1[2]), a_mid, dt, d1[0], d1[1], d1[2]);
              vr = vr + (double)kick_term(FC(d, i2[0], i1[1], i1[2]), a_mid, dt, d2[0], d1[1], d1[2]);
              vr = vr + (double)kick_term(FC(d, i1[0], i2[1], i1[2]), a_mid, dt, d1[0], d2[1], d1[2]);
              vr = vr + (double)kick_term(FC(d, i1[0], i1[1], i2[2]), a_mid, dt, d1[0], d1[1], d2[2]);
              vr = vr + (double)kick_term(FC(d, i1[0], i2[1], i2[2]), a_mid, dt, d1[0], d2[1], d2[2]);
              vr = vr + (double)kick_term(FC(d, i2[0], i1[1], i2[2]), a_mid, dt, d2[0], d1[1], d2[2]);
              vr = vr + (double)kick_term(FC(d, i2[0], i2[1], i1[2]), a_mid, dt, d2[0], d2[1], d1[2]);
              vr = vr + (double)kick_term(FC(d, i2[0], i2[1], i2[2]), a_mid, dt, d2[0], d2[1], d2[2]);
              double sv = vr + (double)bvfield[3 * e + d];
              double a = fabs(sv);
              if (sv > vsg) vsg = sv;
              if (d == 0 && a > v0) v0 = a;
              if (d == 1 && a > v1) v1 = a;
              if (d == 2 && a > v2) v2 = a;
              st_i(bvp, 3 * ip + d, p->izipv, v_encode(vr, c, p->izipv));
            }
#undef FC
          }
        }
    vs = vsg;
    if (v0 > vm[0]) vm[0] = v0;
    if (v1 > vm[1]) vm[1] = v1;
    if (v2 > vm[2]) vm[2] = v2;
  }
  for (int d = 0; d < 3; d++) vmax_out[d] = (float)vm[d];
  if (vmax_signed) *vmax_signed = vs;
}

/* ------------------------------------------------------------------- PP */

/* Short-range particle-particle kick, ext_pp_force (ext_pp_force.f90:36-136),
   in the reference's FP64.  out[0]=f2_max_pp (as real(4)), out[1]=npairs,
   out[2]=itest1 (particles updated). */
void orc_pp_force(const orc_params* p, float a_mid, float dt, float sigma_vi, const int32_t* brhoc,
                  const int64_t* bstart, const void* bxp, void* bvp, double* out, double* fout) {
  int64_t nt = p->nt, nnt = p->nnt, ncell = p->ncell, nft = nt * ncell;
  int64_t pr = p->pp_range;
  int64_t nh = nft + 2 * ncell; /* hoc(1-ncell:nft+ncell)^3 */
  double c = vcoef(sigma_vi);
  double mass = (double)p->mass_p;
  double rsoft = (double)p->rsoft;
  double nfc = (double)p->nf_cutoff;
  int32_t* hoc = (int32_t*)malloc(sizeof(int32_t) * nh * nh * nh);
  double ftemp = 0;
  int64_t npairs = 0, itest1 = 0;
  set_threads(p);
#define HOC(a, b, cc) hoc[((a) + ncell - 1) + nh * (((b) + ncell - 1) + nh * ((cc) + ncell - 1))]
  for (int64_t t = 0; t < nnt * nnt * nnt; t++) {
    if (p->tile_sel >= 0 && t != p->tile_sel) continue;
    int64_t ip_offset = bstart[ext_index(p, 0, 0, 0, t)];
    int64_t e_last = ext_index(p, nt + 1, nt + 1, nt + 1, t);
    int64_t nll = bstart[e_last] + brhoc[e_last] - ip_offset;
    int32_t* ll = (int32_t*)calloc((size_t)(nll + 1), sizeof(int32_t));
    memset(hoc, 0, sizeof(int32_t) * nh * nh * nh);
    /* linked list over fine cells (ext_pp_force.f90:53-75) */
    for (int64_t igz = 0; igz <= nt + 1; igz++)
      for (int64_t igy = 0; igy <= nt + 1; igy++)
        for (int64_t igx = 0; igx <= nt + 1; igx++) {
          int64_t e = ext_index(p, igx, igy, igz, t);
          int64_t cidx[3] = {igx, igy, igz};
          for (int64_t lp = 0; lp < brhoc[e]; lp++) {
            int64_t ip1 = bstart[e] + lp;
            int64_t iv[3];
            for (int d = 0; d < 3; d++) {
              double xv = fine_pos(ncell, cidx[d], ld_i(bxp, 3 * ip1 + d, p->izipx), p->izipx);
              iv[d] = (int64_t)floor(xv) + 1;
            }
            int64_t ipll1 = ip1 - ip_offset + 1;
            ll[ipll1] = HOC(iv[0], iv[1], iv[2]);
            HOC(iv[0], iv[1], iv[2]) = (int32_t)ipll1;
          }
        }
    double ft = ftemp;
    int64_t np_t = 0, it_t = 0;
    /* pair force and kick (ext_pp_force.f90:84-129) */
#pragma omp parallel for schedule(static, 2) reduction(+ : np_t, it_t) reduction(max : ft)
    for (int64_t igz = 1; igz <= nft; igz++)
      for (int64_t igy = 1; igy <= nft; igy++)
        for (int64_t igx = 1; igx <= nft; igx++) {
          int64_t ipll1 = HOC(igx, igy, igz);
          int64_t g1[3] = {igx, igy, igz};
          while (ipll1 != 0) {
            it_t++;
            int64_t ip1 = ipll1 + ip_offset - 1;
            double xv1[3], vr[3], ftot[3] = {0, 0, 0};
            for (int d = 0; d < 3; d++) {
              /* ncell*floor((ig-1)/4.) with the real(4) division (ext_pp_force.f90:91) */
              int64_t cc = (int64_t)floorf((float)(g1[d] - 1) / 4.0f);
              xv1[d] = fine_pos(ncell, cc + 1, ld_i(bxp, 3 * ip1 + d, p->izipx), p->izipx);
              vr[d] = v_decode(ld_i(bvp, 3 * ip1 + d, p->izipv), c, p->izipv);
            }
            for (int64_t kk = igz - pr; kk <= igz + pr; kk++)
              for (int64_t jj = igy - pr; jj <= igy + pr; jj++)
                for (int64_t ii = igx - pr; ii <= igx + pr; ii++) {
                  int64_t ipll2 = HOC(ii, jj, kk);
                  int64_t g2[3] = {ii, jj, kk};
                  while (ipll2 != 0) {
                    np_t++;
                    int64_t ip2 = ipll2 + ip_offset - 1;
                    double x21[3];
                    for (int d = 0; d < 3; d++) {
                      int64_t cc = (int64_t)floorf((float)(g2[d] - 1) / 4.0f);
                      double xv2 = fine_pos(ncell, cc + 1, ld_i(bxp, 3 * ip2 + d, p->izipx), p->izipx);
                      x21[d] = xv2 - xv1[d];
                    }
                    double rmag = sqrt((x21[0] * x21[0] + x21[1] * x21[1]) + x21[2] * x21[2]);
                    if (rmag == 0) rmag = 1.0;
                    double rcut = rmag / nfc;
                    double rc3 = (rcut * rcut) * rcut;
                    double rc2 = rcut * rcut, rc4 = rc2 * rc2, rc5 = rc4 * rcut;
                    double pcut = (1.0 - ((double)1.75f * rc3)) + ((double)0.75f * rc5);
                    double r3 = (rmag * rmag) * rmag;
                    for (int d = 0; d < 3; d++) {
                      double f = (mass * (x21[d] / r3)) * pcut;
                      if (!(rmag > rsoft)) f = f * 0.0;
                      ftot[d] = ftot[d] + f;
                    }
                    ipll2 = ll[ipll2];
                  }
                }
            if (fout)  /* f_tot of this particle, by buffered index (a checking output) */
              for (int d = 0; d < 3; d++) fout[3 * ip1 + d] = ftot[d];
            for (int d = 0; d < 3; d++) {
              double kick = (((ftot[d] * (double)a_mid) * (double)dt) / 6.0) / (double)PI_F;
              vr[d] = vr[d] + kick;
              st_i(bvp, 3 * ip1 + d, p->izipv, v_encode(vr[d], c, p->izipv));
            }
            double f2 = (ftot[0] * ftot[0] + ftot[1] * ftot[1]) + ftot[2] * ftot[2];
            if ((double)(float)f2 > ft) ft = (double)(float)f2;
            ipll1 = ll[ipll1];
          }
        }
    ftemp = ft;
    npairs += np_t;
    itest1 += it_t;
    free(ll);
  }
#undef HOC
  free(hoc);
  out[0] = (double)(float)ftemp;
  out[1] = (double)npairs;
  out[2] = (double)itest1;
}
