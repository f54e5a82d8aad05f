// cube_timing.cu -- per-phase CUDA-event timers on the context's stream.
//
// The reference times each phase with system_clock and prints it
// (pm.f90:35-411, update_particle.f90:31-252, ext_pp_force.f90:40-132).  Here
// every phase is bracketed by a pair of events recorded on the launching
// stream when timing is enabled; pairs are harvested (one synchronisation) on
// cube_timing_read, so enabling timing adds no host synchronisation to a step.
#include <vector>

#include "cube_internal.cuh"

static const char* kPhaseNames[CUBE_NPHASE] = {
    "update_dest", "update_rank", "update_scan", "update_scatter", "update_sigma", "pp_force",
    "fine_deposit", "fine_r2c", "fine_green", "fine_c2r", "fine_f2max", "fine_kick",
    "coarse_deposit", "coarse_fft", "coarse_kick", "update_place"};

struct TimerPair {
  cudaEvent_t a, b;
  int phase;
};

struct CubeTimers {
  std::vector<TimerPair> pool;
  size_t used = 0;
  int open_phase = -1;
  double ms[CUBE_NPHASE] = {0};
  long long cnt[CUBE_NPHASE] = {0};
};

static void harvest(cube_ctx* c) {
  CubeTimers* t = c->timers;
  if (!t || t->used == 0) return;
  cudaEventSynchronize(t->pool[t->used - 1].b);
  for (size_t i = 0; i < t->used; i++) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, t->pool[i].a, t->pool[i].b) == cudaSuccess) {
      t->ms[t->pool[i].phase] += ms;
      t->cnt[t->pool[i].phase] += 1;
    }
  }
  t->used = 0;
}

void cube_phase_begin(cube_ctx* c, int phase) {
  CubeTimers* t = c->timers;
  if (!t) return;
  if (t->used == t->pool.size()) {
    if (t->pool.size() >= 4096) {
      harvest(c);
    } else {
      TimerPair p{};
      cudaEventCreate(&p.a);
      cudaEventCreate(&p.b);
      t->pool.push_back(p);
    }
  }
  t->pool[t->used].phase = phase;
  cudaEventRecord(t->pool[t->used].a, c->stream);
  t->open_phase = phase;
}

void cube_phase_end(cube_ctx* c, int phase) {
  CubeTimers* t = c->timers;
  if (!t || t->open_phase != phase) return;
  cudaEventRecord(t->pool[t->used].b, c->stream);
  t->used++;
  t->open_phase = -1;
}

void cube_timers_free(cube_ctx* c) {
  CubeTimers* t = c->timers;
  if (!t) return;
  for (auto& p : t->pool) {
    cudaEventDestroy(p.a);
    cudaEventDestroy(p.b);
  }
  delete t;
  c->timers = nullptr;
}

extern "C" int cube_timing(cube_ctx* c, int enable) {
  if (!c) return CUBE_ERR_ARG;
  CUBE_CUDA(c, cudaSetDevice(c->device));
  if (enable) {
    if (!c->timers) c->timers = new CubeTimers();
    harvest(c);
    for (int i = 0; i < CUBE_NPHASE; i++) {
      c->timers->ms[i] = 0;
      c->timers->cnt[i] = 0;
    }
  } else {
    cube_timers_free(c);
  }
  return CUBE_OK;
}

extern "C" int cube_timing_read(cube_ctx* c, double* ms, int64_t* count, int nphase) {
  if (!c || nphase < 0) return CUBE_ERR_ARG;
  if (!c->timers) return cube_fail(c, CUBE_ERR_STATE, "timing is not enabled");
  CUBE_CUDA(c, cudaSetDevice(c->device));
  harvest(c);
  for (int i = 0; i < nphase && i < CUBE_NPHASE; i++) {
    if (ms) ms[i] = c->timers->ms[i];
    if (count) count[i] = c->timers->cnt[i];
  }
  return CUBE_OK;
}

extern "C" const char* cube_phase_name(int phase) {
  return (phase >= 0 && phase < CUBE_NPHASE) ? kPhaseNames[phase] : "";
}

extern "C" void* cube_stream(cube_ctx* c) { return c ? (void*)c->stream : nullptr; }
