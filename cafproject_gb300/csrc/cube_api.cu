// cube_api.cu -- the C ABI (include/cube_gpu.h): context life cycle, state
// transfer, field inspection, and the entry points that replace the bodies of
// the reference subroutines update_x, ext_pp_force and particle_mesh.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <vector>

#include "cube_internal.cuh"

int cube_fail(cube_ctx* c, int code, const std::string& msg) {
  if (c) c->err = msg;
  return code;
}

int cube_grid(int64_t work, int block, int max_blocks_per_sm) {
  static int nsm = 0;
  if (nsm == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    if (nsm <= 0) nsm = 152;
  }
  int64_t need = (work + block - 1) / block;
  int64_t cap = (int64_t)nsm * max_blocks_per_sm;
  if (need < 1) need = 1;
  return (int)(need < cap ? need : cap);
}

static int alloc(cube_ctx* c, void** p, size_t bytes) {
  cudaError_t e = cudaMalloc(p, bytes ? bytes : 16);
  if (e != cudaSuccess) {
    return cube_fail(c, CUBE_ERR_NOMEM, std::string("cudaMalloc of ") + std::to_string(bytes) +
                                            " bytes failed: " + cudaGetErrorString(e));
  }
  return CUBE_OK;
}
#define ALLOC(ptr, bytes)                                  \
  do {                                                     \
    int r_ = alloc(c, (void**)&(ptr), (size_t)(bytes));    \
    if (r_) return r_;                                     \
  } while (0)

static void release(cube_ctx* c) {
  if (!c) return;
  cudaSetDevice(c->device);
  if (c->stream_copy) {
    cudaStreamSynchronize(c->stream_copy);
    cudaStreamDestroy(c->stream_copy);
    cudaEventDestroy(c->ev_copy_start);
    cudaEventDestroy(c->ev_copy);
    cudaEventDestroy(c->ev_pid);
  }
  cube_timers_free(c);
  if (c->owner) {  // meshes, kernels, plans, work area and stream belong to the owner
    if (c->owner->linked == c) c->owner->linked = nullptr;
    c->rho_f = c->kern_f = c->kern_f_raw = c->rho_c = c->kern_c = nullptr;
    for (int d = 0; d < 3; d++) c->force_f[d] = c->force_c[d] = nullptr;
    c->cufft_work = nullptr;
    c->plan_f_r2c = c->plan_f_c2r = c->plan_c_r2c = c->plan_c_c2r = 0;
    c->stream = nullptr;
  }
  void* bufs[] = {c->xp[0], c->xp[1], c->vp[0], c->vp[1], c->pid[0], c->pid[1], c->pcell[0], c->pcell[1],
                  c->rhoc[0], c->rhoc[1],
                  c->vfield[0], c->vfield[1], c->cstart[0], c->cstart[1], c->dest, c->dframe, c->doff, c->lrank, c->offc, c->perm, c->vdense, c->rank, c->xtra,
                  c->scan_tmp, c->red_tmp, c->tan_tab, c->codec[0].dec, c->codec[1].dec, c->codec[0].bnd, c->codec[1].bnd, c->codec[0].dech, c->codec[1].dech, c->codec[0].rt, c->codec[1].rt, c->rho_f, c->force_f[0],
                  c->force_f[1], c->force_f[2], c->kern_f, c->kern_f_raw, c->rho_c, c->force_c[0],
                  c->force_c[1], c->force_c[2], c->kern_c, c->fpp, c->pp_list[0], c->pp_list[1], c->pp_list[2], c->pp_list[3], c->pp_list[4], c->pp_scr_pts,
                  c->pp_lpart[0], c->pp_lpart[1], c->pp_lpart[2], c->pp_lpart[3], c->pp_lpart[4], c->pp_nlist, c->dstats,
                  c->pp_occ, c->pp_act, c->pp_wcnt, c->pp_wstart, c->pp_arhoc, c->pp_acstart, c->pp_aidx,
                  c->cufft_work};
  for (void* b : bufs)
    if (b) cudaFree(b);
  for (int i = 0; i < 2; i++) {
    if (c->skey[i]) cudaFree(c->skey[i]);
    if (c->sval[i]) cudaFree(c->sval[i]);
  }
  if (c->sort_tmp) cudaFree(c->sort_tmp);
  if (c->hstats) cudaFreeHost(c->hstats);
  if (c->hstats_pp) cudaFreeHost(c->hstats_pp);
  if (c->dstats_pp) cudaFree(c->dstats_pp);
  if (c->ev_fork) cudaEventDestroy(c->ev_fork);
  if (c->ev_pp) cudaEventDestroy(c->ev_pp);
  if (c->stream_pp) cudaStreamDestroy(c->stream_pp);
  if (c->pp_nlist_host) cudaFreeHost(c->pp_nlist_host);
  if (c->plan_f_r2c) cufftDestroy(c->plan_f_r2c);
  if (c->plan_f_c2r) cufftDestroy(c->plan_f_c2r);
  if (c->plan_c_r2c) cufftDestroy(c->plan_c_r2c);
  if (c->plan_c_c2r) cufftDestroy(c->plan_c_c2r);
  if (c->stream) cudaStreamDestroy(c->stream);
}

static int make_plans(cube_ctx* c) {
  // fine: nf^3 in place, FFTW-compatible padded layout; one shared work area
  size_t wf1 = 0, wf2 = 0, wc1 = 0, wc2 = 0;
  int nf = c->nf, nc = c->p.nc;
  CUBE_FFT(c, cufftCreate(&c->plan_f_r2c));
  CUBE_FFT(c, cufftCreate(&c->plan_f_c2r));
  CUBE_FFT(c, cufftCreate(&c->plan_c_r2c));
  CUBE_FFT(c, cufftCreate(&c->plan_c_c2r));
  for (cufftHandle h : {c->plan_f_r2c, c->plan_f_c2r, c->plan_c_r2c, c->plan_c_c2r})
    CUBE_FFT(c, cufftSetAutoAllocation(h, 0));
  CUBE_FFT(c, cufftMakePlan3d(c->plan_f_r2c, nf, nf, nf, CUFFT_R2C, &wf1));
  CUBE_FFT(c, cufftMakePlan3d(c->plan_f_c2r, nf, nf, nf, CUFFT_C2R, &wf2));
  CUBE_FFT(c, cufftMakePlan3d(c->plan_c_r2c, nc, nc, nc, CUFFT_R2C, &wc1));
  CUBE_FFT(c, cufftMakePlan3d(c->plan_c_c2r, nc, nc, nc, CUFFT_C2R, &wc2));
  size_t w = wf1;
  for (size_t x : {wf2, wc1, wc2})
    if (x > w) w = x;
  c->cufft_work_bytes = w;
  ALLOC(c->cufft_work, w);
  for (cufftHandle h : {c->plan_f_r2c, c->plan_f_c2r, c->plan_c_r2c, c->plan_c_c2r}) {
    CUBE_FFT(c, cufftSetWorkArea(h, c->cufft_work));
    CUBE_FFT(c, cufftSetStream(h, c->stream));
  }
  return CUBE_OK;
}

static int create_impl(const cube_params* p, const float* fine_table, const float* coarse_table, int device,
                       cube_ctx* owner, cube_ctx** out) {
  if (!p || !out || (!owner && (!fine_table || !coarse_table))) return CUBE_ERR_ARG;
  *out = nullptr;
  cube_ctx* c = new (std::nothrow) cube_ctx();
  if (!c) return CUBE_ERR_NOMEM;
  c->p = *p;
  c->device = device;
  auto bad = [&](const char* m) {
    c->err = m;
    *out = c;
    return CUBE_ERR_ARG;
  };
  if (p->nc <= 0 || p->nnt <= 0 || p->nc % p->nnt) return bad("nc must be a positive multiple of nnt");
  // LRCKCORR rescales the coarse modes with |k|<=8 by 1/Im FFT(raw kernel)
  // (kernel_c.f90:111-113); below nc = 16 that sphere wraps past Nyquist
  if (p->nc < 16) return bad("nc must be at least 16 (coarse kernel correction needs |k|<=8 up to Nyquist)");
  // the deposits keep a cell's coordinates in 16-bit fields; far beyond any mesh HBM holds
  if (p->nc > 16384) return bad("nc must be at most 16384");
  if (p->ncell != 4) return bad("ncell must be 4");
  if (p->izipx < 1 || p->izipx > 2 || p->izipv < 1 || p->izipv > 2) return bad("izipx/izipv must be 1 or 2");
  c->nt = p->nc / p->nnt;
  if (c->nt < 2 * p->ncb) return bad("nt must be at least 2*ncb");
  if (p->nf_cutoff >= p->ncb * p->ncell) return bad("nf_cutoff must be below the tile buffer nfb");
  if (p->pp_range != 1 && p->pp_on) return bad("pp_range must be 1");
  if (p->np_max <= 0) return bad("np_max must be positive");
  if (p->ncb < 1 || p->ncb > 8) return bad("ncb must be in 1..8");
  c->nf = p->nc * p->ncell;
  c->ntiles = p->nnt * p->nnt * p->nnt;
  c->ncells = (int64_t)p->nc * p->nc * p->nc;
  c->nfine = (int64_t)c->nf * c->nf * c->nf;
  c->nvbin = 1 << (8 * p->izipv);
  if (owner) {
    const cube_params& q = owner->p;
    if (p->nc != q.nc || p->nnt != q.nnt || p->ncell != q.ncell || p->ncb != q.ncb || p->nf_cutoff != q.nf_cutoff ||
        device != owner->device)
      return bad("a linked species needs the mesh geometry and device of its owner");
    if (owner->owner) return bad("link to the owning context");
    if (p->pp_on) return bad("the linked species takes no PP force");
  }
  *out = c;
  CUBE_CUDA(c, cudaSetDevice(device));
  if (owner) {
    c->owner = owner;
    owner->linked = c;
    c->stream = owner->stream;
  } else {
    CUBE_CUDA(c, cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
  }
  int64_t np = p->np_max;
  for (int k = 0; k < 2; k++) {
    ALLOC(c->xp[k], 3 * np * p->izipx);
    ALLOC(c->vp[k], 3 * np * p->izipv);
    ALLOC(c->pid[k], 4 * np);
    ALLOC(c->pcell[k], 4 * np);
    ALLOC(c->rhoc[k], 4 * c->ncells);
    ALLOC(c->vfield[k], 12 * c->ncells);
    ALLOC(c->cstart[k], 8 * (c->ncells + 1));
  }
  ALLOC(c->dest, 4 * np);
  ALLOC(c->dframe, np);
  ALLOC(c->doff, np);
  ALLOC(c->lrank, 2 * np);
  ALLOC(c->offc, 2 * 27 * c->ncells);
  ALLOC(c->perm, 4 * np);
  ALLOC(c->vdense, 4 * c->ncells);
  ALLOC(c->rank, 4 * np);
  c->xtra_cap = 1 << 20;
  ALLOC(c->xtra, sizeof(int4) * c->xtra_cap);
  // the cell-count scans, and PP's prefilter scan of one count per 32 particles
  c->scan_tmp_bytes = 8 * (std::max<int64_t>(c->ncells, np / 32 + 1) / 256 + 1024);
  ALLOC(c->scan_tmp, c->scan_tmp_bytes);
  c->red_blocks = 2048;
  ALLOC(c->red_tmp, sizeof(double) * 4 * c->red_blocks);
  ALLOC(c->tan_tab, 4 * c->nvbin);
  for (int k = 0; k < 2; k++) {
    ALLOC(c->codec[k].dec, 8 * c->nvbin);
    ALLOC(c->codec[k].dech, 8 * c->nvbin);
    ALLOC(c->codec[k].bnd, 8 * (c->nvbin / 2 + 1));
    ALLOC(c->codec[k].rt, 4 * c->nvbin);
  }
  if (owner) {
    c->rho_f = owner->rho_f;
    c->kern_f = owner->kern_f;
    c->rho_c = owner->rho_c;
    c->kern_c = owner->kern_c;
    for (int d = 0; d < 3; d++) {
      c->force_f[d] = owner->force_f[d];
      c->force_c[d] = owner->force_c[d];
    }
  } else {
    int64_t nfh = (int64_t)(c->nf / 2 + 1);
    int64_t fpad = 2 * nfh * c->nf * (int64_t)c->nf;  // floats of a padded fine mesh
    ALLOC(c->rho_f, 4 * fpad);
    for (int d = 0; d < 3; d++) ALLOC(c->force_f[d], 4 * fpad);
    ALLOC(c->kern_f, 4 * 3 * nfh * c->nf * (int64_t)c->nf);
    int64_t nch = (int64_t)(p->nc / 2 + 1);
    int64_t cpad = 2 * nch * p->nc * (int64_t)p->nc;
    ALLOC(c->rho_c, 4 * cpad);
    for (int d = 0; d < 3; d++) ALLOC(c->force_c[d], 4 * cpad);
    ALLOC(c->kern_c, 4 * 3 * nch * p->nc * (int64_t)p->nc);
  }
  if (p->pp_on) {
    ALLOC(c->fpp, 12 * (size_t)np);
    // PP's global staging for cells too dense for shared memory (24 bytes an
    // entry): a cell and its fine ring stage each particle once when nc >= 3
    // (27 times in a smaller periodic box), and at most 2^22 entries
    c->pp_scr_cap = std::min<int64_t>((p->nc >= 3 ? 1 : 27) * (int64_t)np, (int64_t)1 << 22) + 64;
    ALLOC(c->pp_scr_pts, 24 * (size_t)c->pp_scr_cap);
    const int64_t nw = (np + 31) / 32;
    ALLOC(c->pp_occ, 16 * (size_t)c->ncells);
    ALLOC(c->pp_act, 4 * (size_t)nw);
    ALLOC(c->pp_wcnt, 4 * (size_t)nw);
    ALLOC(c->pp_wstart, 8 * (size_t)(nw + 1));
    ALLOC(c->pp_arhoc, 4 * (size_t)c->ncells);
    ALLOC(c->pp_acstart, 8 * (size_t)(c->ncells + 1));
    ALLOC(c->pp_aidx, 4 * (size_t)np);
    ALLOC(c->dstats_pp, sizeof(DevStats));
    CUBE_CUDA(c, cudaMallocHost((void**)&c->hstats_pp, sizeof(DevStats)));
    // PP beside the PM force chain at the higher priority: its blocks take
    // free SM slots first while the transforms stream (74.4 against 75.2 ms
    // a 512^3 step; the other way round, 77.2)
    int prio_lo = 0, prio_hi = 0;
    CUBE_CUDA(c, cudaDeviceGetStreamPriorityRange(&prio_lo, &prio_hi));
    CUBE_CUDA(c, cudaStreamCreateWithPriority(&c->stream_pp, cudaStreamNonBlocking, prio_hi));
    CUBE_CUDA(c, cudaEventCreateWithFlags(&c->ev_fork, cudaEventDisableTiming));
    CUBE_CUDA(c, cudaEventCreateWithFlags(&c->ev_pp, cudaEventDisableTiming));
    int r = cube_pp_init(c);
    if (r) return r;
  }
  {
    int nb = (p->nc + 3) / 4;
    c->pp_brick_cap = nb * nb * nb;
    for (int l = 0; l < 5; l++) {
      const size_t cap = l < 2 ? (size_t)c->pp_brick_cap : (size_t)c->ncells;
      ALLOC(c->pp_list[l], 4 * cap);
      ALLOC(c->pp_lpart[l], 4 * cap);
    }
    ALLOC(c->pp_nlist, 64);
    CUBE_CUDA(c, cudaMallocHost((void**)&c->pp_nlist_host, 32));
    for (int l = 0; l < 5; l++) c->pp_nlist_host[l] = 0;
  }
  ALLOC(c->dstats, sizeof(DevStats));
  CUBE_CUDA(c, cudaMallocHost((void**)&c->hstats, sizeof(DevStats)));
  int r;
  if (owner) {
    c->plan_f_r2c = owner->plan_f_r2c;
    c->plan_f_c2r = owner->plan_f_c2r;
    c->plan_c_r2c = owner->plan_c_r2c;
    c->plan_c_c2r = owner->plan_c_c2r;
    c->cufft_work = owner->cufft_work;
    c->cufft_work_bytes = owner->cufft_work_bytes;
  } else {
    r = make_plans(c);
    if (r) return r;
  }
  r = cube_build_tables(c);
  if (r) return r;
  if (!owner) {
    r = cube_kernels_init(c, fine_table, coarse_table);
    if (r) return r;
  }
  CUBE_CUDA(c, cudaStreamSynchronize(c->stream));
  return CUBE_OK;
}

extern "C" int cube_create(const cube_params* p, const float* fine_table, const float* coarse_table, int device,
                           cube_ctx** out) {
  return create_impl(p, fine_table, coarse_table, device, nullptr, out);
}

extern "C" int cube_create_linked(const cube_params* p, cube_ctx* owner, cube_ctx** out) {
  if (!owner) return CUBE_ERR_ARG;
  return create_impl(p, nullptr, nullptr, owner->device, owner, out);
}

extern "C" int cube_destroy(cube_ctx* c) {
  if (!c) return CUBE_ERR_ARG;
  release(c);
  delete c;
  return CUBE_OK;
}

extern "C" const char* cube_last_error(const cube_ctx* c) { return c ? c->err.c_str() : "null context"; }

extern "C" int cube_upload_state(cube_ctx* c, int64_t nplocal, const void* xp, const void* vp, const int32_t* pid,
                                 const int32_t* rhoc, const float* vfield) {
  if (!c || !xp || !vp || !rhoc || !vfield || nplocal < 0) return CUBE_ERR_ARG;
  if (nplocal > c->p.np_max) return cube_fail(c, CUBE_ERR_IMAGE_OVERFLOW, "nplocal exceeds np_max");
  CUBE_CUDA(c, cudaSetDevice(c->device));
  return cube_state_in(c, nplocal, xp, vp, pid, rhoc, vfield);
}

extern "C" int cube_download_state(cube_ctx* c, int64_t* nplocal, void* xp, void* vp, int32_t* pid, int32_t* rhoc,
                                   float* vfield) {
  if (!c) return CUBE_ERR_ARG;
  if (!c->have_state) return cube_fail(c, CUBE_ERR_STATE, "no state uploaded");
  CUBE_CUDA(c, cudaSetDevice(c->device));
  return cube_state_out(c, nplocal, xp, vp, pid, rhoc, vfield);
}

extern "C" int cube_upload_begin(cube_ctx* c, int64_t nplocal, const void* xp, const void* vp, const int32_t* pid,
                                 const int32_t* rhoc, const float* vfield) {
  if (!c || !xp || !vp || !rhoc || !vfield || nplocal < 0) return CUBE_ERR_ARG;
  if (nplocal > c->p.np_max) return cube_fail(c, CUBE_ERR_IMAGE_OVERFLOW, "nplocal exceeds np_max");
  CUBE_CUDA(c, cudaSetDevice(c->device));
  return cube_state_in(c, nplocal, xp, vp, pid, rhoc, vfield, true);
}

extern "C" int cube_download_begin(cube_ctx* c, int64_t* nplocal, void* xp, void* vp, int32_t* pid, int32_t* rhoc,
                                   float* vfield) {
  if (!c) return CUBE_ERR_ARG;
  if (!c->have_state) return cube_fail(c, CUBE_ERR_STATE, "no state uploaded");
  if (c->copy_pending) return cube_fail(c, CUBE_ERR_STATE, "a download is already in flight");
  CUBE_CUDA(c, cudaSetDevice(c->device));
  return cube_state_out_begin(c, nplocal, xp, vp, pid, rhoc, vfield);
}

extern "C" int cube_download_finish(cube_ctx* c) {
  if (!c) return CUBE_ERR_ARG;
  CUBE_CUDA(c, cudaSetDevice(c->device));
  return cube_state_out_finish(c);
}

extern "C" int cube_set_sigma(cube_ctx* c, float s, float sn) {
  if (!c) return CUBE_ERR_ARG;
  c->sigma_vi = s;
  c->sigma_vi_new = sn;
  return CUBE_OK;
}

extern "C" int cube_get_sigma(const cube_ctx* c, float* s, float* sn) {
  if (!c) return CUBE_ERR_ARG;
  if (s) *s = c->sigma_vi;
  if (sn) *sn = c->sigma_vi_new;
  return CUBE_OK;
}

// join: order the context stream after a pending cube_upload_begin first
// (cube_update_x takes the pieces as they land instead)
static int check_ready(cube_ctx* c, bool join = true) {
  if (!c) return CUBE_ERR_ARG;
  if (!c->have_state) return cube_fail(c, CUBE_ERR_STATE, "no state uploaded");
  CUBE_CUDA(c, cudaSetDevice(c->device));
  return join ? cube_upload_join(c) : CUBE_OK;
}

extern "C" int cube_update_x(cube_ctx* c, float dt_old, float dt, float vz_max, cube_stats* st) {
  int r = check_ready(c, false);
  if (!r) r = cube_copy_join(c);
  if (r) return r;
  return cube_update_x_impl(c, dt_old, dt, vz_max, st);
}

extern "C" int cube_buffer_grid(cube_ctx* c) { return check_ready(c); }
extern "C" int cube_buffer_x(cube_ctx* c) { return check_ready(c); }
extern "C" int cube_buffer_v(cube_ctx* c) { return check_ready(c); }

extern "C" int cube_pp_force(cube_ctx* c, float a_mid, float dt, cube_stats* st) {
  int r = check_ready(c);
  if (r) return r;
  return cube_pp_impl(c, a_mid, dt, st);
}

extern "C" int cube_pm_fine_density(cube_ctx* c, cube_stats* st) {
  int r = check_ready(c);
  if (r) return r;
  return cube_fine_density_impl(c, st);
}
extern "C" int cube_pm_coarse_density(cube_ctx* c, cube_stats* st) {
  int r = check_ready(c);
  if (r) return r;
  return cube_coarse_density_impl(c, st);
}
extern "C" int cube_pm_fine_forces(cube_ctx* c, cube_stats* st) {
  int r = check_ready(c);
  if (r) return r;
  return cube_fine_forces_impl(c, st);
}
extern "C" int cube_pm_fine_kick(cube_ctx* c, float a_mid, float dt) {
  int r = check_ready(c);
  if (r) return r;
  return cube_fine_kick_impl(c, a_mid, dt);
}
extern "C" int cube_pm_coarse_forces(cube_ctx* c, cube_stats* st) {
  int r = check_ready(c);
  if (r) return r;
  return cube_coarse_forces_impl(c, st);
}
extern "C" int cube_pm_coarse_kick(cube_ctx* c, float a_mid, float dt, cube_stats* st) {
  int r = check_ready(c);
  if (r) return r;
  return cube_coarse_kick_impl(c, a_mid, dt, st);
}

extern "C" int cube_particle_mesh(cube_ctx* c, float a_mid, float dt, cube_stats* st) {
  int r = check_ready(c);
  if (r) return r;
  const float pre[2] = {a_mid, dt};
  if ((r = cube_fine_forces_impl(c, st, pre))) return r;
  if ((r = cube_fine_kick_impl(c, a_mid, dt, true))) return r;
  c->sigma_vi = c->sigma_vi_new;  // pm.f90:193
  if ((r = cube_coarse_forces_impl(c, st, pre))) return r;
  return cube_coarse_kick_impl(c, a_mid, dt, st, true);
}

// ext_pp_force followed by particle_mesh (main.f90:113-116) with PP on a
// second stream beside the PM force chain: the fine and coarse densities,
// transforms and maxima need only positions, so they run while PP kicks;
// the fine kick waits for PP's kick, as in the reference's order.  Same
// results, bit for bit, as the two calls made one after the other.
extern "C" int cube_pp_particle_mesh(cube_ctx* c, float a_mid, float dt, cube_stats* st_pp, cube_stats* st_pm) {
  int r = check_ready(c);
  if (r) return r;
  if (!c->stream_pp) return cube_fail(c, CUBE_ERR_ARG, "PP is off for this context (pp_on = 0)");
  const float pre[2] = {a_mid, dt};
  CUBE_CUDA(c, cudaEventRecord(c->ev_fork, c->stream));
  CUBE_CUDA(c, cudaStreamWaitEvent(c->stream_pp, c->ev_fork, 0));
  {  // PP's launches go to its stream with its own stats
    cudaStream_t s0 = c->stream;
    DevStats *d0 = c->dstats, *h0 = c->hstats;
    c->stream = c->stream_pp;
    c->dstats = c->dstats_pp;
    c->hstats = c->hstats_pp;
    r = cube_pp_launch(c, a_mid, dt, /*defer_kick=*/true);
    if (!r) r = cudaEventRecord(c->ev_pp, c->stream_pp) == cudaSuccess ? CUBE_OK : CUBE_ERR_CUDA;
    c->stream = s0;
    c->dstats = d0;
    c->hstats = h0;
    if (r) return r;
  }
  if ((r = cube_fine_forces_impl(c, st_pm, pre))) return r;
  if ((r = cube_coarse_forces_impl(c, st_pm, pre))) return r;
  CUBE_CUDA(c, cudaStreamWaitEvent(c->stream, c->ev_pp, 0));
  // the fine kick applies PP's kick first (ext_pp_force.f90:116-121), then its own
  if ((r = cube_fine_kick_impl(c, a_mid, dt, true, /*with_pp=*/true))) return r;
  c->sigma_vi = c->sigma_vi_new;  // pm.f90:193
  if ((r = cube_coarse_kick_impl(c, a_mid, dt, st_pm, true))) return r;
  {  // PP's stats (its stream is done: the kicks waited for it)
    cudaStream_t s0 = c->stream;
    DevStats *d0 = c->dstats, *h0 = c->hstats;
    c->stream = c->stream_pp;
    c->dstats = c->dstats_pp;
    c->hstats = c->hstats_pp;
    r = cube_pp_finish(c, st_pp);
    c->stream = s0;
    c->dstats = d0;
    c->hstats = h0;
  }
  return r;
}

// particle_mesh with the linked species (pm.f90:52-107, 162-189, 237-253,
// 358-377): both species deposit into the same meshes, both are kicked by the
// same forces with their own velocity codes; vmax is reported per species.
extern "C" int cube_particle_mesh2(cube_ctx* c, cube_ctx* nu, float a_mid, float dt, cube_stats* st,
                                   cube_stats* st_nu) {
  int r = check_ready(c);
  if (r) return r;
  if (!nu || nu->owner != c) return cube_fail(c, CUBE_ERR_ARG, "the second species must be linked to this context");
  if (!nu->have_state) return cube_fail(c, CUBE_ERR_STATE, "no state uploaded for the linked species");
  if ((r = cube_upload_join(nu))) return cube_fail(c, r, nu->err);
  const float pre[2] = {a_mid, dt};
  if ((r = cube_fine_density_impl(c, nullptr, false))) return r;
  if ((r = cube_fine_density_impl(nu, nullptr, true))) return cube_fail(c, r, nu->err);
  if ((r = cube_fine_spectral_impl(c, st, pre))) return r;
  if ((r = cube_fine_kick_impl(c, a_mid, dt, true))) return r;
  if ((r = cube_fine_kick_impl(nu, a_mid, dt, true))) return cube_fail(c, r, nu->err);
  c->sigma_vi = c->sigma_vi_new;  // pm.f90:193-194
  nu->sigma_vi = nu->sigma_vi_new;
  if ((r = cube_coarse_density_impl(c, nullptr, false))) return r;
  if ((r = cube_coarse_density_impl(nu, nullptr, true))) return cube_fail(c, r, nu->err);
  if ((r = cube_coarse_spectral_impl(c, st, pre))) return r;
  if ((r = cube_coarse_kick_impl(c, a_mid, dt, st, true))) return r;
  if ((r = cube_coarse_kick_impl(nu, a_mid, dt, st_nu, true))) return cube_fail(c, r, nu->err);
  // testrhof / testrhoc sum both species' mass (pm.f90:108, 258); the coarse
  // kick left the second species' deposited masses in its host stats
  if (st) {
    st->testrhof += std::ldexp((double)nu->hstats->rhof_fix, -dep_shift(nu->p.mass_p));
    st->testrhoc += std::ldexp((double)nu->hstats->rhoc_fix, -dep_shift(nu->p.mass_p));
  }
  return CUBE_OK;
}

// Density stages of cube_particle_mesh2, for parity tests: both species'
// CIC deposits into the shared fine (coarse) mesh, testrhof (testrhoc) the
// total mass.
static int density2(cube_ctx* c, cube_ctx* nu, cube_stats* st, bool fine) {
  int r = check_ready(c);
  if (r) return r;
  if (!nu || nu->owner != c) return cube_fail(c, CUBE_ERR_ARG, "the second species must be linked to this context");
  if (!nu->have_state) return cube_fail(c, CUBE_ERR_STATE, "no state uploaded for the linked species");
  if ((r = cube_upload_join(nu))) return cube_fail(c, r, nu->err);
  cube_stats a{}, b{};
  if ((r = fine ? cube_fine_density_impl(c, &a, false) : cube_coarse_density_impl(c, &a, false))) return r;
  if ((r = fine ? cube_fine_density_impl(nu, &b, true) : cube_coarse_density_impl(nu, &b, true)))
    return cube_fail(c, r, nu->err);
  if (st) {
    st->testrhof = a.testrhof + b.testrhof;
    st->testrhoc = a.testrhoc + b.testrhoc;
  }
  return CUBE_OK;
}
extern "C" int cube_pm_fine_density2(cube_ctx* c, cube_ctx* nu, cube_stats* st) { return density2(c, nu, st, true); }
extern "C" int cube_pm_coarse_density2(cube_ctx* c, cube_ctx* nu, cube_stats* st) {
  return density2(c, nu, st, false);
}

extern "C" int64_t cube_nplocal(const cube_ctx* c) { return c ? c->np : -1; }

extern "C" int cube_set_option(cube_ctx* c, int option, int64_t value) {
  if (!c) return CUBE_ERR_ARG;
  switch (option) {
    case CUBE_OPT_EXACT_KICKS:
      c->opt_exact_kicks = value ? 1 : 0;
      return CUBE_OK;
    case CUBE_OPT_RANK_WALK:
      if (value < 0 || value > 2) return cube_fail(c, CUBE_ERR_ARG, "rank path is 0, 1 or 2");
      c->opt_rank_walk = (int)value;
      return CUBE_OK;
    case CUBE_OPT_PP_LEVEL:
      if (value < 0 || value > 5) return cube_fail(c, CUBE_ERR_ARG, "PP level must be 0 to 5");
      c->opt_pp_level = (int)value;
      return CUBE_OK;
    case CUBE_OPT_PP_HEAVY:
      if (value < 0 || value > (1 << 30)) return cube_fail(c, CUBE_ERR_ARG, "PP warp-walk threshold out of range");
      c->opt_pp_heavy = (int)value;
      return CUBE_OK;
    case CUBE_OPT_PP_PARTS:
      if (value < 0 || value > 255) return cube_fail(c, CUBE_ERR_ARG, "PP parts must be 0 to 255");
      c->opt_pp_parts = (int)value;
      return CUBE_OK;
    case CUBE_OPT_PP_FILTER:
      if (value < 0 || value > 2) return cube_fail(c, CUBE_ERR_ARG, "PP prefilter is 0 (automatic), 1 (off) or 2 (on)");
      c->opt_pp_filter = (int)value;
      return CUBE_OK;
    case CUBE_OPT_DEPOSIT_FINE:
    case CUBE_OPT_DEPOSIT_COARSE:
      if (value < 0 || value > 3) return cube_fail(c, CUBE_ERR_ARG, "deposit brick shape must be 0 to 3");
      (option == CUBE_OPT_DEPOSIT_FINE ? c->opt_dep_fine : c->opt_dep_coarse) = (int)value;
      return CUBE_OK;
    case CUBE_OPT_FAIL_ALLOC:
      if (value < 0 || value > 64) return cube_fail(c, CUBE_ERR_ARG, "allocation fault index must be 0 to 64");
      c->fail_alloc = (int)value;
      return CUBE_OK;
    default:
      return cube_fail(c, CUBE_ERR_ARG, "unknown option");
  }
}

extern "C" int cube_synchronize(cube_ctx* c) {
  if (!c) return CUBE_ERR_ARG;
  CUBE_CUDA(c, cudaSetDevice(c->device));
  CUBE_CUDA(c, cudaStreamSynchronize(c->stream));
  if (c->stream_copy) CUBE_CUDA(c, cudaStreamSynchronize(c->stream_copy));
  return CUBE_OK;
}

// ------------------------------------------------------------------ fields
// Copy between a dense host array and a padded device mesh (row stride n+2).
static int mesh_copy(cube_ctx* c, float* dev, int n, void* host, bool to_host) {
  size_t row = (size_t)n * 4, dpitch = (size_t)(n + 2) * 4;
  size_t rows = (size_t)n * n;
  if (to_host)
    CUBE_CUDA(c, cudaMemcpy2DAsync(host, row, dev, dpitch, row, rows, cudaMemcpyDeviceToHost, c->stream));
  else
    CUBE_CUDA(c, cudaMemcpy2DAsync(dev, dpitch, host, row, row, rows, cudaMemcpyHostToDevice, c->stream));
  CUBE_CUDA(c, cudaStreamSynchronize(c->stream));
  return CUBE_OK;
}

static int field_io(cube_ctx* c, int field, void* host, bool to_host) {
  if (!c || !host) return CUBE_ERR_ARG;
  CUBE_CUDA(c, cudaSetDevice(c->device));
  int nf = c->nf, nc = c->p.nc;
  switch (field) {
    case CUBE_FIELD_RHO_F:
      return mesh_copy(c, c->rho_f, nf, host, to_host);
    case CUBE_FIELD_FORCE_F:
      for (int d = 0; d < 3; d++) {
        int r = mesh_copy(c, c->force_f[d], nf, (char*)host + (size_t)d * 4 * c->nfine, to_host);
        if (r) return r;
      }
      return CUBE_OK;
    case CUBE_FIELD_RHO_C:
      return mesh_copy(c, c->rho_c, nc, host, to_host);
    case CUBE_FIELD_FORCE_C:
      for (int d = 0; d < 3; d++) {
        int r = mesh_copy(c, c->force_c[d], nc, (char*)host + (size_t)d * 4 * c->ncells, to_host);
        if (r) return r;
      }
      return CUBE_OK;
    case CUBE_FIELD_KERN_F:
    case CUBE_FIELD_KERN_C: {
      if (!to_host) return cube_fail(c, CUBE_ERR_ARG, "kernels are read-only");
      bool fine = field == CUBE_FIELD_KERN_F;
      int n = fine ? nf : nc;
      size_t cnt = 3 * (size_t)(n / 2 + 1) * n * n;
      CUBE_CUDA(c, cudaMemcpyAsync(host, fine ? c->kern_f : c->kern_c, cnt * 4, cudaMemcpyDeviceToHost, c->stream));
      CUBE_CUDA(c, cudaStreamSynchronize(c->stream));
      // undo the folded 1/n^3 normalisation
      double s = (double)n * n * n;
      float* h = (float*)host;
      for (size_t i = 0; i < cnt; i++) h[i] = (float)((double)h[i] * s);
      return CUBE_OK;
    }
    case CUBE_FIELD_FORCE_PP: {
      if (!to_host) return cube_fail(c, CUBE_ERR_ARG, "the PP force is read-only");
      if (!c->fpp) return cube_fail(c, CUBE_ERR_ARG, "PP is off for this context (pp_on = 0)");
      if (!c->have_state) return cube_fail(c, CUBE_ERR_STATE, "no state uploaded");
      CUBE_CUDA(c, cudaMemcpyAsync(host, c->fpp, 12 * (size_t)c->np, cudaMemcpyDeviceToHost, c->stream));
      if (c->pp_act_valid) {
        // a filtered call wrote the active particles' forces only: the others' are zero
        std::vector<unsigned> act((size_t)((c->np + 31) / 32));
        CUBE_CUDA(c, cudaMemcpyAsync(act.data(), c->pp_act, 4 * act.size(), cudaMemcpyDeviceToHost, c->stream));
        CUBE_CUDA(c, cudaStreamSynchronize(c->stream));
        float* f = (float*)host;
        for (int64_t p = 0; p < c->np; p++)
          if (!((act[(size_t)(p >> 5)] >> (p & 31)) & 1u)) f[3 * p] = f[3 * p + 1] = f[3 * p + 2] = 0.f;
        return CUBE_OK;
      }
      CUBE_CUDA(c, cudaStreamSynchronize(c->stream));
      return CUBE_OK;
    }
    default:
      return cube_fail(c, CUBE_ERR_ARG, "unknown field");
  }
}

extern "C" int cube_get_field(cube_ctx* c, int field, void* host) { return field_io(c, field, host, true); }
extern "C" int cube_set_field(cube_ctx* c, int field, const void* host) {
  return field_io(c, field, const_cast<void*>(host), false);
}
