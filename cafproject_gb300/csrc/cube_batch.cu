// cube_batch.cu -- an ensemble of independent boxes (each its own CUBE image:
// own particle count, cosmology, seed and step schedule) advanced together.
//
// Every box is a full context of the plain path.  In graph mode the whole
// step of every box -- update_x, ext_pp_force, particle_mesh, exactly the
// plain path's kernels -- is one captured CUDA graph with one branch per box,
// launched once per step:
//   head    k_batch_head (per box): the step's scalars from the box's
//           schedule and the previous step's results, with the eager host
//           path's arithmetic (update_particle.f90:32,37; ext_pp_force.f90:94;
//           the coarse kick's exact-vmax threshold);
//   step    update_x with the rank-path choice, the extra-copy count and
//           sigma_vi_new resolved on the device, PP, particle_mesh;
//   tail    k_batch_tail: vmax / vz_max / sigma carried to the next step, the
//           step's stats appended to a device history; codec slot 1
//           (sigma_vi_new) copied to slot 0.
// The state buffers of a context alternate between steps, so two graphs are
// captured (even and odd steps).  No host synchronisation happens between
// steps; the host reads the history when it asks for it.  Serial mode runs the
// same schedule through the eager entry points, one box after another -- the
// plain form run in sequence, which graph mode must reproduce bit for bit.
//
// The step schedule (dt and a_mid per step, dt_old = 0 before the first) is
// the caller's: the reference's timestep derives it from force maxima
// (timestep.f90), which would put the host back inside every step; an
// ensemble runs a fixed schedule per box instead.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "cube_internal.cuh"

struct cube_batch {
  int device = 0, mode = 0, nbox = 0, nsteps = 0;
  std::vector<cube_ctx*> box;
  std::vector<int> pp_level;
  std::vector<float> vz;         // serial mode: sim%vz_max per box (host)
  std::vector<cube_batch_stats> hhist;  // serial mode: per step and box
  cudaStream_t s0 = nullptr;
  StepDev* sd = nullptr;         // nbox
  StepOut* sout = nullptr;       // nbox
  StepOut* hist = nullptr;       // nsteps x nbox
  float2* sched = nullptr;       // nbox x nsteps (dt, a_mid)
  std::vector<float2> hsched;
  cudaGraphExec_t g[2] = {nullptr, nullptr};
  struct Snap {
    int cur;
    void* vp[2];
  };
  std::vector<Snap> snap[2];     // each context's buffers after graph p
  cudaEvent_t fork = nullptr, t0 = nullptr, t1 = nullptr;
  std::vector<cudaEvent_t> join;
  int64_t steps_done = 0;
  float last_ms = 0.f, last_dev_ms = 0.f;  // wall clock / device time of the last cube_batch_step
  std::vector<float> step_ms;              // per step: device time (graph) or wall clock (serial)
  std::string err;
};

namespace {

int bfail(cube_batch* b, int code, const std::string& m) {
  if (b) b->err = m;
  return code;
}
#define BCUDA(b, call)                                                              \
  do {                                                                              \
    cudaError_t e_ = (call);                                                        \
    if (e_ != cudaSuccess) return bfail(b, CUBE_ERR_CUDA, std::string(#call ": ") + cudaGetErrorString(e_)); \
  } while (0)

// per box, at the head of a step: the eager path's host arithmetic on the device
__global__ void k_batch_head(StepDev* sd, const float2* __restrict__ sched, int nsteps, int ncell) {
  if (threadIdx.x != 0) return;
  const int i = sd->istep;
  const int j = i < nsteps ? i : nsteps - 1;
  const float dt = sched[j].x, a_mid = sched[j].y;
  const float dt_old = j > 0 ? sched[j - 1].x : 0.f;
  StepHost& h = sd->h;
  h.dt = dt;
  h.a_mid = a_mid;
  h.dt_mid = __fdiv_rn(__fadd_rn(dt_old, dt), 2.0f);                      // update_particle.f90:32
  const float q2 = __fdiv_rn(__fmul_rn(h.dt_mid, sd->vz_max), (float)ncell);  // :37, real(4)
  int nl = 2 * (int)ceil((double)q2) + 1;
  h.nlayer = nl < 1 ? 1 : nl;
  for (int d = 0; d < 3; d++) h.tau[d] = __fmul_rn(kVmaxTau, sd->vmax_prev[d]);
  h.kick = __ddiv_rn(__ddiv_rn(__dmul_rn((double)a_mid, (double)dt), 6.0), (double)CUBE_PI_F);
  h.kick_f = __double2float_rn(h.kick);
  h.cf_vi = __double2float_rn(vcoef(sd->sigma_vi));
}

// per box, at the tail: carry vmax, vz_max and sigma, append the stats
__global__ void k_batch_tail(StepDev* sd, StepOut* sout, StepOut* hist, int nbox, int box, int nsteps) {
  if (threadIdx.x != 0) return;
  const DevStats& cs = sout->coarse;
  for (int d = 0; d < 3; d++) sd->vmax_prev[d] = __uint_as_float(cs.vmax_bits[d]);
  sd->vz_max = sd->vmax_prev[2];
  sd->sigma_vi = sd->sigma_new;
  const int i = sd->istep;
  if (i < nsteps) hist[(size_t)i * nbox + box] = *sout;
  sd->istep = i + 1;
}

// the pointer state of a context (what a step changes on the host side)
cube_batch::Snap snap_of(const cube_ctx* c) { return cube_batch::Snap{c->cur, {c->vp[0], c->vp[1]}}; }
void restore(cube_ctx* c, const cube_batch::Snap& s) {
  c->cur = s.cur;
  c->vp[0] = s.vp[0];
  c->vp[1] = s.vp[1];
}

int box_step(cube_ctx* c, int ncell, const float2* sched, int nsteps) {
  k_batch_head<<<1, 32, 0, c->stream>>>(c->sd, sched, nsteps, ncell);
  CUBE_CUDA(c, cudaGetLastError());
  int r = cube_update_x_impl(c, 0.f, 0.f, 0.f, nullptr);
  if (r) return r;
  if (c->p.pp_on && (r = cube_pp_impl(c, 0.f, 0.f, nullptr))) return r;
  const float pre[2] = {0.f, 0.f};
  if ((r = cube_fine_forces_impl(c, nullptr, pre))) return r;
  if ((r = cube_fine_kick_impl(c, 0.f, 0.f, true))) return r;
  if ((r = cube_coarse_forces_impl(c, nullptr, pre))) return r;
  return cube_coarse_kick_impl(c, 0.f, 0.f, nullptr, true);
}

int capture(cube_batch* b, int parity) {
  cudaGraph_t g = nullptr;
  BCUDA(b, cudaStreamBeginCapture(b->s0, cudaStreamCaptureModeRelaxed));
  int r = CUBE_OK;
  cudaError_t e = cudaEventRecord(b->fork, b->s0);
  for (int i = 0; i < b->nbox && !r && e == cudaSuccess; i++) {
    cube_ctx* c = b->box[i];
    e = cudaStreamWaitEvent(c->stream, b->fork, 0);
    if (e != cudaSuccess) break;
    r = box_step(c, c->p.ncell, b->sched + (size_t)i * b->nsteps, b->nsteps);
    if (r) {
      b->err = "box " + std::to_string(i) + ": " + c->err;
      break;
    }
    const size_t nv = (size_t)c->nvbin;
    e = cudaMemcpyAsync(c->codec[0].dec, c->codec[1].dec, 8 * nv, cudaMemcpyDeviceToDevice, c->stream);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(c->codec[0].dech, c->codec[1].dech, 8 * nv, cudaMemcpyDeviceToDevice, c->stream);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(c->codec[0].bnd, c->codec[1].bnd, 8 * (nv / 2 + 1), cudaMemcpyDeviceToDevice, c->stream);
    if (e != cudaSuccess) break;
    k_batch_tail<<<1, 32, 0, c->stream>>>(c->sd, c->sout, b->hist, b->nbox, i, b->nsteps);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaEventRecord(b->join[i], c->stream);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(b->s0, b->join[i], 0);
  }
  cudaError_t e2 = cudaStreamEndCapture(b->s0, &g);
  if (r || e != cudaSuccess || e2 != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    if (r) return r;
    return bfail(b, CUBE_ERR_CUDA,
                 std::string("batch capture: ") + cudaGetErrorString(e != cudaSuccess ? e : e2));
  }
  e = cudaGraphInstantiate(&b->g[parity], g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return bfail(b, CUBE_ERR_CUDA, std::string("batch instantiate: ") + cudaGetErrorString(e));
  b->snap[parity].resize(b->nbox);
  for (int i = 0; i < b->nbox; i++) b->snap[parity][i] = snap_of(b->box[i]);
  return CUBE_OK;
}

void drop_graphs(cube_batch* b) {
  for (cudaGraphExec_t& g : b->g)
    if (g) {
      cudaGraphExecDestroy(g);
      g = nullptr;
    }
}

void release(cube_batch* b) {
  cudaSetDevice(b->device);
  drop_graphs(b);
  for (cube_ctx* c : b->box)
    if (c) {
      c->sd = nullptr;
      c->sout = nullptr;
      c->graph_mode = false;
      cube_destroy(c);
    }
  for (void* p : {(void*)b->sd, (void*)b->sout, (void*)b->hist, (void*)b->sched})
    if (p) cudaFree(p);
  for (cudaEvent_t e : b->join)
    if (e) cudaEventDestroy(e);
  for (cudaEvent_t e : {b->fork, b->t0, b->t1})
    if (e) cudaEventDestroy(e);
  if (b->s0) cudaStreamDestroy(b->s0);
}

}  // namespace

extern "C" int cube_batch_create(const cube_batch_box* boxes, int nbox, const float* fine_table,
                                 const float* coarse_table, int device, int mode, cube_batch** out) {
  if (!boxes || nbox < 1 || !fine_table || !coarse_table || !out) return CUBE_ERR_ARG;
  if (mode != CUBE_BATCH_GRAPH && mode != CUBE_BATCH_SERIAL) return CUBE_ERR_ARG;
  *out = nullptr;
  cube_batch* b = new (std::nothrow) cube_batch();
  if (!b) return CUBE_ERR_NOMEM;
  *out = b;
  b->device = device;
  b->mode = mode;
  b->nbox = nbox;
  BCUDA(b, cudaSetDevice(device));
  BCUDA(b, cudaStreamCreateWithFlags(&b->s0, cudaStreamNonBlocking));
  BCUDA(b, cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming));
  BCUDA(b, cudaEventCreate(&b->t0));
  BCUDA(b, cudaEventCreate(&b->t1));
  b->join.assign(nbox, nullptr);
  for (cudaEvent_t& e : b->join) BCUDA(b, cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  BCUDA(b, cudaMalloc(&b->sd, sizeof(StepDev) * nbox));
  BCUDA(b, cudaMalloc(&b->sout, sizeof(StepOut) * nbox));
  BCUDA(b, cudaMemset(b->sd, 0, sizeof(StepDev) * nbox));
  BCUDA(b, cudaMemset(b->sout, 0, sizeof(StepOut) * nbox));
  b->box.assign(nbox, nullptr);
  b->pp_level.assign(nbox, 0);
  b->vz.assign(nbox, 0.f);
  for (int i = 0; i < nbox; i++) {
    const cube_batch_box& d = boxes[i];
    if (d.params.nnt != 1) return bfail(b, CUBE_ERR_ARG, "batch boxes are single-tile images (nnt = 1)");
    cube_ctx* c = nullptr;
    int r = cube_create(&d.params, fine_table, coarse_table, device, &c);
    b->box[i] = c;
    if (r) return bfail(b, r, "box " + std::to_string(i) + ": " + (c ? c->err : std::string("create failed")));
    float sig = 0.f, vm[3] = {0.f, 0.f, 0.f};
    r = cube_ic_zeldovich(c, &d.cosmo, d.z_init, d.seed, &sig, vm);
    if (r) return bfail(b, r, "box " + std::to_string(i) + " initial conditions: " + c->err);
    // the device-carried state of the first step
    StepDev s0{};
    s0.sigma_vi = sig;
    s0.vz_max = vm[2];
    BCUDA(b, cudaMemcpy(b->sd + i, &s0, sizeof s0, cudaMemcpyHostToDevice));
    c->sd = b->sd + i;
    c->sout = b->sout + i;
    b->vz[i] = vm[2];
  }
  return CUBE_OK;
}

extern "C" int cube_batch_set_schedule(cube_batch* b, int nsteps, const float* dt, const float* a_mid) {
  if (!b || nsteps < 1 || !dt || !a_mid) return CUBE_ERR_ARG;
  BCUDA(b, cudaSetDevice(b->device));
  if (b->steps_done) return bfail(b, CUBE_ERR_STATE, "the schedule is fixed once the boxes have stepped");
  drop_graphs(b);
  b->nsteps = nsteps;
  b->hsched.resize((size_t)b->nbox * nsteps);
  for (size_t i = 0; i < b->hsched.size(); i++) b->hsched[i] = make_float2(dt[i], a_mid[i]);
  if (b->sched) cudaFree(b->sched);
  if (b->hist) cudaFree(b->hist);
  b->sched = nullptr;
  b->hist = nullptr;
  BCUDA(b, cudaMalloc(&b->sched, sizeof(float2) * b->hsched.size()));
  BCUDA(b, cudaMemcpy(b->sched, b->hsched.data(), sizeof(float2) * b->hsched.size(), cudaMemcpyHostToDevice));
  BCUDA(b, cudaMalloc(&b->hist, sizeof(StepOut) * (size_t)nsteps * b->nbox));
  BCUDA(b, cudaMemset(b->hist, 0, sizeof(StepOut) * (size_t)nsteps * b->nbox));
  return CUBE_OK;
}

namespace {

cube_batch_stats stats_of(const StepOut& o) {
  cube_batch_stats s{};
  s.sigma_vi_new = o.sigma_new;
  s.f2_max_fine = bits_float(o.coarse.f2_fine_bits);
  s.f2_max_coarse = bits_float(o.coarse.f2_coarse_bits);
  s.f2_max_pp = bits_float(o.pp.f2_pp_bits);
  for (int d = 0; d < 3; d++) s.vmax[d] = bits_float(o.coarse.vmax_bits[d]);
  s.flags = o.upd.flags;
  s.npairs = (int64_t)o.pp.npairs;
  s.itest1 = (int64_t)o.pp.itest1;
  s.ndup = (int64_t)o.upd.ndup_list;
  s.sum_r = o.sums[1];
  return s;
}

int check_stats(cube_batch* b, int i, int k, const cube_batch_stats& s) {
  const cube_ctx* c = b->box[i];
  const std::string where = "box " + std::to_string(i) + " step " + std::to_string(k + 1) + ": ";
  if (s.flags & 1) return bfail(b, CUBE_ERR_DISPLACEMENT, where + "a particle left the double-buffer tile");
  if (s.flags & 2) return bfail(b, CUBE_ERR_COUNT_MISMATCH, where + "a re-sorted particle had no rank");
  if (s.ndup > c->xtra_cap) return bfail(b, CUBE_ERR_TILE_OVERFLOW, where + "extra-copy list overflow");
  if (c->p.pp_on && s.itest1 != c->np)
    return bfail(b, CUBE_ERR_COUNT_MISMATCH, where + "PP updated a different number of particles than nplocal");
  if (!(s.sigma_vi_new > 0.f)) return bfail(b, CUBE_ERR_NONFINITE, where + "sigma_vi_new is not positive");
  return CUBE_OK;
}

int graph_steps(cube_batch* b, int n) {
  if (!b->g[0]) {
    for (int i = 0; i < b->nbox; i++) {
      cube_ctx* c = b->box[i];
      // codec slot 0 holds the tables of the state's sigma before the first graph step
      int r = cube_codec_build_dev(c, 0, &c->sd->sigma_vi);
      if (r) return bfail(b, r, c->err);
      BCUDA(b, cudaStreamSynchronize(c->stream));
    }
    for (int p = 0; p < 2; p++) {
      for (cube_ctx* c : b->box) c->graph_mode = true;
      int r = capture(b, p);
      for (cube_ctx* c : b->box) c->graph_mode = false;
      if (r) return r;
    }
  }
  const int64_t k0 = b->steps_done;
  // an event between consecutive graph launches gives each step's device time
  std::vector<cudaEvent_t> ev(n + 1, nullptr);
  struct Events {
    std::vector<cudaEvent_t>& v;
    ~Events() {
      for (cudaEvent_t e : v)
        if (e) cudaEventDestroy(e);
    }
  } evs{ev};
  for (cudaEvent_t& e : ev) BCUDA(b, cudaEventCreate(&e));
  BCUDA(b, cudaDeviceSynchronize());
  const auto w0 = std::chrono::steady_clock::now();
  BCUDA(b, cudaEventRecord(ev[0], b->s0));
  for (int k = 0; k < n; k++) {
    BCUDA(b, cudaGraphLaunch(b->g[(k0 + k) & 1], b->s0));
    BCUDA(b, cudaEventRecord(ev[k + 1], b->s0));
  }
  BCUDA(b, cudaStreamSynchronize(b->s0));
  b->last_ms = std::chrono::duration<float, std::milli>(std::chrono::steady_clock::now() - w0).count();
  BCUDA(b, cudaEventElapsedTime(&b->last_dev_ms, ev[0], ev[n]));
  b->step_ms.resize((size_t)b->nsteps, 0.f);
  for (int k = 0; k < n; k++) BCUDA(b, cudaEventElapsedTime(&b->step_ms[(size_t)(k0 + k)], ev[k], ev[k + 1]));
  b->steps_done = k0 + n;
  // the host's view of each context after an even or odd number of graph steps
  const int last = (int)((b->steps_done - 1) & 1);
  std::vector<StepDev> hs(b->nbox);
  BCUDA(b, cudaMemcpy(hs.data(), b->sd, sizeof(StepDev) * b->nbox, cudaMemcpyDeviceToHost));
  for (int i = 0; i < b->nbox; i++) {
    cube_ctx* c = b->box[i];
    restore(c, b->snap[last][i]);
    c->sigma_vi = c->sigma_vi_new = hs[i].sigma_vi;
    for (int d = 0; d < 3; d++) c->vmax_prev[d] = hs[i].vmax_prev[d];
    c->codec[0].sigma = c->codec[1].sigma = hs[i].sigma_vi;
  }
  std::vector<StepOut> ho((size_t)n * b->nbox);
  BCUDA(b, cudaMemcpy(ho.data(), b->hist + (size_t)k0 * b->nbox, sizeof(StepOut) * ho.size(),
                      cudaMemcpyDeviceToHost));
  for (int k = 0; k < n; k++)
    for (int i = 0; i < b->nbox; i++) {
      const cube_batch_stats s = stats_of(ho[(size_t)k * b->nbox + i]);
      b->hhist[(size_t)(k0 + k) * b->nbox + i] = s;
      int r = check_stats(b, i, (int)(k0 + k), s);
      if (r) return r;
    }
  return CUBE_OK;
}

// the plain form, one box after another, through the eager entry points
int serial_steps(cube_batch* b, int n) {
  const int64_t k0 = b->steps_done;
  BCUDA(b, cudaDeviceSynchronize());
  const auto w0 = std::chrono::steady_clock::now();
  b->step_ms.resize((size_t)b->nsteps, 0.f);
  for (int i = 0; i < b->nbox; i++) {
    cube_ctx* c = b->box[i];
    const float2* s = b->hsched.data() + (size_t)i * b->nsteps;
    for (int64_t k = k0; k < k0 + n; k++) {
      const auto ws = std::chrono::steady_clock::now();
      const float dt = s[k].x, a_mid = s[k].y, dt_old = k > 0 ? s[k - 1].x : 0.f;
      cube_stats su{}, sp{}, sm{};
      int r = cube_update_x(c, dt_old, dt, b->vz[i], &su);
      if (!r) r = cube_buffer_grid(c);
      if (!r) r = cube_buffer_x(c);
      if (!r && c->p.pp_on) r = cube_pp_force(c, a_mid, dt, &sp);
      if (!r) r = cube_particle_mesh(c, a_mid, dt, &sm);
      if (!r) r = cube_buffer_v(c);
      if (r) return bfail(b, r, "box " + std::to_string(i) + " step " + std::to_string(k + 1) + ": " + c->err);
      b->vz[i] = sm.vmax[2];  // pm.f90:398
      cube_batch_stats& o = b->hhist[(size_t)k * b->nbox + i];
      o = cube_batch_stats{};
      o.sigma_vi_new = su.sigma_vi_new;
      o.f2_max_fine = sm.f2_max_fine;
      o.f2_max_coarse = sm.f2_max_coarse;
      o.f2_max_pp = sp.f2_max_pp;
      for (int d = 0; d < 3; d++) o.vmax[d] = sm.vmax[d];
      o.npairs = sp.npairs;
      o.itest1 = sp.itest1;
      o.ndup = su.ndup;
      o.sum_r = su.sum_r;
      b->step_ms[(size_t)k] += std::chrono::duration<float, std::milli>(std::chrono::steady_clock::now() - ws).count();
    }
  }
  BCUDA(b, cudaDeviceSynchronize());
  b->last_ms = std::chrono::duration<float, std::milli>(std::chrono::steady_clock::now() - w0).count();
  b->last_dev_ms = b->last_ms;
  b->steps_done = k0 + n;
  return CUBE_OK;
}

}  // namespace

extern "C" int cube_batch_step(cube_batch* b, int nsteps) {
  if (!b || nsteps < 0) return CUBE_ERR_ARG;
  BCUDA(b, cudaSetDevice(b->device));
  if (!b->nsteps) return bfail(b, CUBE_ERR_STATE, "no schedule set");
  if (b->steps_done + nsteps > b->nsteps) return bfail(b, CUBE_ERR_ARG, "steps beyond the schedule");
  if (nsteps == 0) return CUBE_OK;
  if (b->hhist.size() != (size_t)b->nsteps * b->nbox) b->hhist.assign((size_t)b->nsteps * b->nbox, cube_batch_stats{});
  for (cube_ctx* c : b->box)  // host copies of a box's state started through its context end first
    if (c->stream_copy) {
      BCUDA(b, cudaStreamSynchronize(c->stream_copy));
      c->copy_pending = c->pid_pending = c->xv_pending = false;
    }
  return b->mode == CUBE_BATCH_GRAPH ? graph_steps(b, nsteps) : serial_steps(b, nsteps);
}

namespace {

// device time of f() on c's stream: the median of three runs after one
float time_on(cube_batch* b, cube_ctx* c, int (*f)(cube_ctx*), int* err) {
  float t[4] = {0, 0, 0, 0};
  for (int rep = 0; rep < 4; rep++) {
    if (cudaEventRecord(b->t0, c->stream) != cudaSuccess || (*err = f(c)) ||
        cudaEventRecord(b->t1, c->stream) != cudaSuccess || cudaEventSynchronize(b->t1) != cudaSuccess ||
        cudaEventElapsedTime(&t[rep], b->t0, b->t1) != cudaSuccess) {
      if (!*err) *err = CUBE_ERR_CUDA;
      return 0.f;
    }
  }
  std::sort(t + 1, t + 4);
  return t[2];
}
int fine_density_only(cube_ctx* c) { return cube_fine_density_impl(c, nullptr, false); }
int coarse_density_only(cube_ctx* c) { return cube_coarse_density_impl(c, nullptr, false); }

}  // namespace

extern "C" int cube_batch_autotune(cube_batch* b, int32_t* choices) {
  if (!b) return CUBE_ERR_ARG;
  BCUDA(b, cudaSetDevice(b->device));
  if (b->steps_done || b->g[0]) return bfail(b, CUBE_ERR_STATE, "tune before the first step");
  // per distinct box geometry, on the first such box's initial state and by
  // device time: the fine and coarse deposits' brick shapes (their shared-
  // memory tiles), then the PP start level (which staging tiles carry the
  // pairs).  Every choice gives bitwise the same results; only time depends
  // on it.  The deposits leave the particles alone; PP kicks them, so its
  // trials run on a copy of the state that is put back afterwards.
  std::vector<int> done(b->nbox, 0);
  for (int i = 0; i < b->nbox; i++) {
    if (done[i]) continue;
    cube_ctx* c = b->box[i];
    int err = 0;
    int best_f = 0, best_c = 0, best_pp = 0;
    float bf = 1e30f, bc = 1e30f;
    for (int v = 0; v < 4; v++) {
      c->opt_dep_fine = v;
      const float t = time_on(b, c, fine_density_only, &err);
      if (err) return bfail(b, err, c->err);
      if (t < bf) {
        bf = t;
        best_f = v;
      }
      c->opt_dep_coarse = v;
      const float u = time_on(b, c, coarse_density_only, &err);
      if (err) return bfail(b, err, c->err);
      if (u < bc) {
        bc = u;
        best_c = v;
      }
    }
    if (c->p.pp_on) {
      const int64_t np = c->np;
      std::vector<char> xp(3 * (size_t)np * c->p.izipx), vp(3 * (size_t)np * c->p.izipv);
      std::vector<int32_t> pid(np), rhoc(c->ncells);
      std::vector<float> vf(3 * (size_t)c->ncells);
      int64_t n = 0;
      int r = cube_download_state(c, &n, xp.data(), vp.data(), pid.data(), rhoc.data(), vf.data());
      if (r) return bfail(b, r, c->err);
      float bestms = 1e30f;
      for (int lev = 0; lev <= 4; lev++) {
        float ms = 0.f;
        for (int rep = 0; rep < 3; rep++) {
          if ((r = cube_upload_state(c, n, xp.data(), vp.data(), pid.data(), rhoc.data(), vf.data())))
            return bfail(b, r, c->err);
          c->opt_pp_level = lev;
          BCUDA(b, cudaEventRecord(b->t0, c->stream));
          if ((r = cube_pp_force(c, 0.01f, 0.01f, nullptr))) return bfail(b, r, c->err);
          BCUDA(b, cudaEventRecord(b->t1, c->stream));
          BCUDA(b, cudaEventSynchronize(b->t1));
          float t = 0.f;
          BCUDA(b, cudaEventElapsedTime(&t, b->t0, b->t1));
          if (rep) ms += t;  // the first run warms the caches
        }
        if (ms < bestms) {
          bestms = ms;
          best_pp = lev;
        }
      }
      if ((r = cube_upload_state(c, n, xp.data(), vp.data(), pid.data(), rhoc.data(), vf.data())))
        return bfail(b, r, c->err);
    }
    for (int j = i; j < b->nbox; j++) {
      cube_ctx* q = b->box[j];
      if (!done[j] && q->p.nc == c->p.nc && q->p.pp_on == c->p.pp_on) {
        q->opt_pp_level = best_pp;
        q->opt_dep_fine = best_f;
        q->opt_dep_coarse = best_c;
        b->pp_level[j] = best_pp;
        done[j] = 1;
      }
    }
  }
  if (choices)
    for (int i = 0; i < b->nbox; i++) {
      choices[3 * i] = b->box[i]->opt_pp_level;
      choices[3 * i + 1] = b->box[i]->opt_dep_fine;
      choices[3 * i + 2] = b->box[i]->opt_dep_coarse;
    }
  return CUBE_OK;
}

extern "C" int cube_batch_history(cube_batch* b, int step, cube_batch_stats* out) {
  if (!b || !out || step < 0 || step >= b->steps_done) return CUBE_ERR_ARG;
  for (int i = 0; i < b->nbox; i++) out[i] = b->hhist[(size_t)step * b->nbox + i];
  return CUBE_OK;
}

extern "C" int cube_batch_ctx(cube_batch* b, int box, cube_ctx** ctx) {
  if (!b || !ctx || box < 0 || box >= b->nbox) return CUBE_ERR_ARG;
  *ctx = b->box[box];
  return CUBE_OK;
}

extern "C" int cube_batch_time(const cube_batch* b, float* last_ms, float* last_dev_ms, int64_t* steps_done) {
  if (!b) return CUBE_ERR_ARG;
  if (last_ms) *last_ms = b->last_ms;
  if (last_dev_ms) *last_dev_ms = b->last_dev_ms;
  if (steps_done) *steps_done = b->steps_done;
  return CUBE_OK;
}

extern "C" int cube_batch_step_times(const cube_batch* b, float* ms) {
  if (!b || !ms) return CUBE_ERR_ARG;
  for (int64_t k = 0; k < b->steps_done; k++) ms[k] = k < (int64_t)b->step_ms.size() ? b->step_ms[(size_t)k] : 0.f;
  return CUBE_OK;
}

extern "C" const char* cube_batch_last_error(const cube_batch* b) { return b ? b->err.c_str() : "null batch"; }

extern "C" int cube_batch_destroy(cube_batch* b) {
  if (!b) return CUBE_ERR_ARG;
  release(b);
  delete b;
  return CUBE_OK;
}
