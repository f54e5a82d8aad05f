// cube_state.cu -- state upload/download, the per-particle cell index, the
// velocity-code tables, the deterministic exclusive scan (the spine of
// variables.f90:96-211) and the statistics read-back.
#include <cmath>
#include <mutex>
#include <vector>

#include "cube_internal.cuh"

// ------------------------------------------------------------------ scan
// Exclusive scan of int32 counts into int64 starts[0..n] (starts[n] = total),
// three passes with a fixed block partition so the result never depends on
// scheduling: block sums, one-block scan of the sums, block-local scan + offset.
constexpr int SCAN_T = 256;
constexpr int SCAN_I = 16;
constexpr int SCAN_CHUNK = SCAN_T * SCAN_I;

__device__ __forceinline__ long long warp_incl_scan(long long v) {
  for (int o = 1; o < 32; o <<= 1) {
    long long n = __shfl_up_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) >= o) v += n;
  }
  return v;
}
// block-wide exclusive scan of one value per thread; returns the block total
__device__ long long block_excl_scan(long long v, long long* s_warp, long long& total) {
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  long long inc = warp_incl_scan(v);
  if (lane == 31) s_warp[w] = inc;
  __syncthreads();
  if (w == 0) {
    long long t = lane < nw ? s_warp[lane] : 0;
    long long ti = warp_incl_scan(t);
    if (lane < nw) s_warp[lane] = ti - t;
    if (lane == nw - 1) s_warp[32] = ti;
  }
  __syncthreads();
  long long r = inc - v + s_warp[w];
  total = s_warp[32];
  __syncthreads();
  return r;
}

__global__ void k_scan_blocksum(const int32_t* __restrict__ cnt, int64_t n, long long* __restrict__ bsum) {
  __shared__ long long s[33];
  int64_t base = (int64_t)blockIdx.x * SCAN_CHUNK;
  long long v = 0;
  for (int i = 0; i < SCAN_I; i++) {
    int64_t k = base + (int64_t)i * SCAN_T + threadIdx.x;
    if (k < n) v += cnt[k];
  }
  long long tot;
  block_excl_scan(v, s, tot);
  if (threadIdx.x == 0) bsum[blockIdx.x] = tot;
}

__global__ void k_scan_sums(long long* __restrict__ bsum, int64_t nb) {
  __shared__ long long s[33];
  long long carry = 0;
  for (int64_t b0 = 0; b0 < nb; b0 += blockDim.x) {
    int64_t k = b0 + threadIdx.x;
    long long v = k < nb ? bsum[k] : 0;
    long long tot;
    long long e = block_excl_scan(v, s, tot);
    if (k < nb) bsum[k] = e + carry;
    carry += tot;
  }
}

__global__ void k_scan_final(const int32_t* __restrict__ cnt, int64_t n, const long long* __restrict__ bsum,
                             int64_t* __restrict__ starts) {
  __shared__ long long s[33];
  __shared__ int32_t tile[SCAN_CHUNK];
  int64_t base = (int64_t)blockIdx.x * SCAN_CHUNK;
  for (int i = threadIdx.x; i < SCAN_CHUNK; i += SCAN_T) {
    int64_t k = base + i;
    tile[i] = k < n ? cnt[k] : 0;
  }
  __syncthreads();
  long long v = 0;
  for (int i = 0; i < SCAN_I; i++) v += tile[threadIdx.x * SCAN_I + i];
  long long tot;
  long long run = block_excl_scan(v, s, tot) + bsum[blockIdx.x];
  for (int i = 0; i < SCAN_I; i++) {
    int64_t k = base + (int64_t)threadIdx.x * SCAN_I + i;
    if (k < n) starts[k] = run;
    run += tile[threadIdx.x * SCAN_I + i];
    if (k == n - 1) starts[n] = run;
  }
}

int cube_scan_counts(cube_ctx* c, const int32_t* counts, int64_t* starts, int64_t n) {
  int64_t nb = (n + SCAN_CHUNK - 1) / SCAN_CHUNK;
  if ((size_t)nb * 8 > c->scan_tmp_bytes) return cube_fail(c, CUBE_ERR_ARG, "scan scratch too small");
  long long* bsum = (long long*)c->scan_tmp;
  k_scan_blocksum<<<(unsigned)nb, SCAN_T, 0, c->stream>>>(counts, n, bsum);
  k_scan_sums<<<1, 1024, 0, c->stream>>>(bsum, nb);
  k_scan_final<<<(unsigned)nb, SCAN_T, 0, c->stream>>>(counts, n, bsum, starts);
  CUBE_CUDA(c, cudaGetLastError());
  return CUBE_OK;
}

// ---------------------------------------------------------- cell index
// pcell[p] = cell of particle p, from the spine: one thread per cell; a
// negative count is flagged (bit 16 of *flags) and writes nothing.
__global__ void k_fill_pcell(const int32_t* __restrict__ rhoc, const int64_t* __restrict__ cstart, int64_t ncells,
                             int32_t* __restrict__ pcell, int* flags) {
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < ncells; c += (int64_t)gridDim.x * blockDim.x) {
    if (rhoc && rhoc[c] < 0) {
      atomicOr(flags, 1 << 16);
      continue;
    }
    for (int64_t p = cstart[c]; p < cstart[c + 1]; p++) pcell[p] = (int32_t)c;
  }
}

int cube_state_in(cube_ctx* c, int64_t np, const void* xp, const void* vp, const int32_t* pid, const int32_t* rhoc,
                  const float* vfield, bool defer) {
  int k = c->cur;
  const cube_params& p = c->p;
  int r = cube_copy_join(c);
  if (!r) r = cube_upload_join(c);
  if (r) return r;
  // the counts are checked on the device, after the copies (a failed check
  // leaves the context without a state)
  c->have_state = false;
  CUBE_CUDA(c, cudaMemcpyAsync(c->rhoc[k], rhoc, (size_t)4 * c->ncells, cudaMemcpyHostToDevice, c->stream));
  if (defer) {
    // vfield, then xp and vp piece by piece, then pid on the copy stream: the
    // re-sort's first pass takes each piece as it lands (cube_update_x); the
    // count check below needs only rhoc
    if ((r = cube_copy_stream(c))) return r;
    cudaStream_t s = c->stream_copy;
    CUBE_CUDA(c, cudaEventRecord(c->ev_copy_start, c->stream));
    CUBE_CUDA(c, cudaStreamWaitEvent(s, c->ev_copy_start, 0));
    CUBE_CUDA(c, cudaMemcpyAsync(c->vfield[k], vfield, (size_t)12 * c->ncells, cudaMemcpyHostToDevice, s));
    const size_t bx = 3 * (size_t)p.izipx, bv = 3 * (size_t)p.izipv;
    for (int i = 0; i < cube_ctx::UP_PIECES; i++) {
      const int64_t p0 = np * i / cube_ctx::UP_PIECES, p1 = np * (i + 1) / cube_ctx::UP_PIECES;
      CUBE_CUDA(c, cudaMemcpyAsync((char*)c->xp[k] + bx * p0, (const char*)xp + bx * p0, bx * (p1 - p0),
                                   cudaMemcpyHostToDevice, s));
      CUBE_CUDA(c, cudaMemcpyAsync((char*)c->vp[k] + bv * p0, (const char*)vp + bv * p0, bv * (p1 - p0),
                                   cudaMemcpyHostToDevice, s));
      CUBE_CUDA(c, cudaEventRecord(c->ev_xv[i], s));
    }
    if (pid)
      CUBE_CUDA(c, cudaMemcpyAsync(c->pid[k], pid, (size_t)4 * np, cudaMemcpyHostToDevice, s));
    else
      CUBE_CUDA(c, cudaMemsetAsync(c->pid[k], 0, (size_t)4 * np, s));
    CUBE_CUDA(c, cudaEventRecord(c->ev_pid, s));
    c->xv_pending = c->pid_pending = true;
    c->up_np = np;
  } else {
    CUBE_CUDA(c, cudaMemcpyAsync(c->xp[k], xp, (size_t)3 * np * p.izipx, cudaMemcpyHostToDevice, c->stream));
    CUBE_CUDA(c, cudaMemcpyAsync(c->vp[k], vp, (size_t)3 * np * p.izipv, cudaMemcpyHostToDevice, c->stream));
    if (pid)
      CUBE_CUDA(c, cudaMemcpyAsync(c->pid[k], pid, (size_t)4 * np, cudaMemcpyHostToDevice, c->stream));
    else
      CUBE_CUDA(c, cudaMemsetAsync(c->pid[k], 0, (size_t)4 * np, c->stream));
    CUBE_CUDA(c, cudaMemcpyAsync(c->vfield[k], vfield, (size_t)12 * c->ncells, cudaMemcpyHostToDevice, c->stream));
  }
  r = cube_scan_counts(c, c->rhoc[k], c->cstart[k], c->ncells);
  if (r) return r;
  CUBE_CUDA(c, cudaMemsetAsync(&c->dstats->flags, 0, sizeof(int), c->stream));
  k_fill_pcell<<<cube_grid(c->ncells, 256), 256, 0, c->stream>>>(c->rhoc[k], c->cstart[k], c->ncells, c->pcell[k],
                                                                 &c->dstats->flags);
  CUBE_CUDA(c, cudaGetLastError());
  int64_t tot = -1;
  int fl = 0;
  CUBE_CUDA(c, cudaMemcpyAsync(&tot, c->cstart[k] + c->ncells, 8, cudaMemcpyDeviceToHost, c->stream));
  CUBE_CUDA(c, cudaMemcpyAsync(&fl, &c->dstats->flags, 4, cudaMemcpyDeviceToHost, c->stream));
  CUBE_CUDA(c, cudaStreamSynchronize(c->stream));
  if ((fl & (1 << 16)) || tot != np) {
    if (defer) {  // no state: the pieces still in flight end before the call does
      CUBE_CUDA(c, cudaStreamSynchronize(c->stream_copy));
      c->xv_pending = c->pid_pending = false;
    }
    if (fl & (1 << 16)) return cube_fail(c, CUBE_ERR_ARG, "negative rhoc");
    return cube_fail(c, CUBE_ERR_COUNT_MISMATCH, "sum(rhoc) != nplocal");
  }
  c->np = np;
  c->npglobal = np;
  c->have_state = true;
  for (int d = 0; d < 3; d++) c->vmax_prev[d] = 0.f;
  return CUBE_OK;
}

int cube_state_out(cube_ctx* c, int64_t* np, void* xp, void* vp, int32_t* pid, int32_t* rhoc, float* vfield) {
  int k = c->cur;
  const cube_params& p = c->p;
  if (int r = cube_upload_join(c)) return r;
  if (np) *np = c->np;
  if (xp) CUBE_CUDA(c, cudaMemcpyAsync(xp, c->xp[k], (size_t)3 * c->np * p.izipx, cudaMemcpyDeviceToHost, c->stream));
  if (vp) CUBE_CUDA(c, cudaMemcpyAsync(vp, c->vp[k], (size_t)3 * c->np * p.izipv, cudaMemcpyDeviceToHost, c->stream));
  if (pid) CUBE_CUDA(c, cudaMemcpyAsync(pid, c->pid[k], (size_t)4 * c->np, cudaMemcpyDeviceToHost, c->stream));
  if (rhoc) CUBE_CUDA(c, cudaMemcpyAsync(rhoc, c->rhoc[k], (size_t)4 * c->ncells, cudaMemcpyDeviceToHost, c->stream));
  if (vfield)
    CUBE_CUDA(c, cudaMemcpyAsync(vfield, c->vfield[k], (size_t)12 * c->ncells, cudaMemcpyDeviceToHost, c->stream));
  CUBE_CUDA(c, cudaStreamSynchronize(c->stream));
  return CUBE_OK;
}

int cube_copy_stream(cube_ctx* c) {
  if (c->stream_copy) return CUBE_OK;
  CUBE_CUDA(c, cudaStreamCreateWithFlags(&c->stream_copy, cudaStreamNonBlocking));
  CUBE_CUDA(c, cudaEventCreateWithFlags(&c->ev_copy_start, cudaEventDisableTiming));
  CUBE_CUDA(c, cudaEventCreateWithFlags(&c->ev_copy, cudaEventDisableTiming));
  CUBE_CUDA(c, cudaEventCreateWithFlags(&c->ev_pid, cudaEventDisableTiming));
  for (int i = 0; i < cube_ctx::UP_PIECES; i++)
    CUBE_CUDA(c, cudaEventCreateWithFlags(&c->ev_xv[i], cudaEventDisableTiming));
  return CUBE_OK;
}

int cube_copy_join(cube_ctx* c) {
  if (c->copy_pending) CUBE_CUDA(c, cudaStreamWaitEvent(c->stream, c->ev_copy, 0));
  return CUBE_OK;
}

int cube_pid_join(cube_ctx* c) {
  if (c->pid_pending) {
    CUBE_CUDA(c, cudaStreamWaitEvent(c->stream, c->ev_pid, 0));
    c->pid_pending = false;
  }
  return CUBE_OK;
}

int cube_upload_join(cube_ctx* c) {
  if (c->xv_pending) c->pid_pending = true;  // pid is the last piece on the copy stream
  c->xv_pending = false;
  return cube_pid_join(c);
}

// The force half of a step (PP and PM) reads xp, pid, rhoc and vfield and
// writes only vp, so those four can travel to the host while it runs: the
// copies go on their own stream after an event on the context stream.  vp
// follows the next coarse kick, piece by piece (cube_pm_coarse_kick), or the
// finish when no kick comes first.
int cube_state_out_begin(cube_ctx* c, int64_t* np, void* xp, void* vp, int32_t* pid, int32_t* rhoc, float* vfield) {
  int k = c->cur;
  const cube_params& p = c->p;
  if (int r = cube_copy_stream(c)) return r;
  if (np) *np = c->np;
  cudaStream_t s = c->stream_copy;  // a deferred pid upload is earlier on this stream
  CUBE_CUDA(c, cudaEventRecord(c->ev_copy_start, c->stream));
  CUBE_CUDA(c, cudaStreamWaitEvent(s, c->ev_copy_start, 0));
  if (xp) CUBE_CUDA(c, cudaMemcpyAsync(xp, c->xp[k], (size_t)3 * c->np * p.izipx, cudaMemcpyDeviceToHost, s));
  if (pid) CUBE_CUDA(c, cudaMemcpyAsync(pid, c->pid[k], (size_t)4 * c->np, cudaMemcpyDeviceToHost, s));
  if (rhoc) CUBE_CUDA(c, cudaMemcpyAsync(rhoc, c->rhoc[k], (size_t)4 * c->ncells, cudaMemcpyDeviceToHost, s));
  if (vfield) CUBE_CUDA(c, cudaMemcpyAsync(vfield, c->vfield[k], (size_t)12 * c->ncells, cudaMemcpyDeviceToHost, s));
  CUBE_CUDA(c, cudaEventRecord(c->ev_copy, s));
  c->copy_pending = true;
  c->vp_host = vp;
  return CUBE_OK;
}

int cube_state_out_finish(cube_ctx* c) {
  if (c->vp_host) {
    CUBE_CUDA(c, cudaMemcpyAsync(c->vp_host, c->vp[c->cur], (size_t)3 * c->np * c->p.izipv, cudaMemcpyDeviceToHost,
                                 c->stream));
    c->vp_host = nullptr;
  }
  CUBE_CUDA(c, cudaStreamSynchronize(c->stream));
  if (c->copy_pending) {
    CUBE_CUDA(c, cudaEventSynchronize(c->ev_copy));
    c->copy_pending = false;
  }
  return CUBE_OK;
}

// ------------------------------------------------------ velocity tables
// tan_tab[v + nvbin/2] = real(4) tan(pi*real(v)/real(nvbin-1)), the decode of
// update_particle.f90:67, taken as the correctly rounded float(tan(double)).
int cube_build_tables(cube_ctx* c) {
  int nv = c->nvbin;
  std::vector<float> t(nv);
  float nvm1 = (float)(nv - 1);
  for (int i = 0; i < nv; i++) {
    int v = i - nv / 2;
    volatile float a = CUBE_PI_F * (float)v;  // real(4) product, then real(4) quotient
    volatile float arg = a / nvm1;
    t[i] = (float)std::tan((double)arg);
  }
  CUBE_CUDA(c, cudaMemcpyAsync(c->tan_tab, t.data(), 4 * (size_t)nv, cudaMemcpyHostToDevice, c->stream));
  CUBE_CUDA(c, cudaStreamSynchronize(c->stream));
  return CUBE_OK;
}

// sigp, when set, supplies sigma from the device (graph mode)
__global__ void k_decode_table(const float* __restrict__ tan_tab, int nv, float sigma, const float* sigp,
                               double* __restrict__ dec, float2* __restrict__ dech) {
  if (sigp) sigma = *sigp;
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < nv) {
    double d = __ddiv_rn((double)tan_tab[i], vcoef(sigma));
    dec[i] = d;
    float hi = __double2float_rn(d);
    dech[i] = make_float2(hi, __double2float_rn(__dsub_rn(d, (double)hi)));
  }
}

// bnd[n] = bit pattern of the smallest double a >= 0 with
// u(a) = real(nvbin-1)*atan(vcoef*a)/pi >= n - 0.5, i.e. where nint(u) reaches n
// (update_particle.f90:117).  Bisection over the ordered non-negative doubles,
// keeping u(lo) < n - 0.5 <= u(hi): u(0) = 0 < 0.5 and u(+inf) =
// (nvbin-1)/2 * pi/pi_f > nvbin/2 - 1.5.  The bracket starts from the
// closed-form inverse tan(thr*pi/(nvbin-1))/vcoef (a few ulps off) and widens
// geometrically until it holds, so a boundary costs about a dozen FP64 atan
// evaluations instead of 64; the result is the same smallest double.
__device__ __forceinline__ double enc_u(long long bits, double c, int nvbin) {
  return __ddiv_rn(__dmul_rn((double)(nvbin - 1), atan(__dmul_rn(c, __longlong_as_double(bits)))), (double)CUBE_PI_F);
}
__global__ void k_encode_bounds(float sigma, const float* sigp, int nvbin, long long* __restrict__ bnd) {
  if (sigp) sigma = *sigp;
  int n = blockIdx.x * blockDim.x + threadIdx.x + 1;
  int nmax = nvbin / 2 - 1;
  if (n == 1) bnd[0] = 0;
  if (n > nmax) return;
  double c = vcoef(sigma);
  double thr = (double)n - 0.5;
  const long long kInf = 0x7ff0000000000000LL;
  long long lo = 0, hi = kInf;
  const double a = tan(thr * (double)CUBE_PI_F / (double)(nvbin - 1)) / c;
  if (a > 0.0 && a < 1.0e300) {
    const long long g = __double_as_longlong(a);
    long long step = 16;
    if (enc_u(g, c, nvbin) >= thr) {
      hi = g;
      for (int it = 0; it < 40; it++) {
        const long long t = g - step;
        if (t <= 0) break;
        if (enc_u(t, c, nvbin) < thr) {
          lo = t;
          break;
        }
        hi = t;
        step *= 4;
      }
    } else {
      lo = g;
      for (int it = 0; it < 40; it++) {
        const long long t = g + step;
        if (t >= kInf) break;
        if (enc_u(t, c, nvbin) >= thr) {
          hi = t;
          break;
        }
        lo = t;
        step *= 4;
      }
    }
  }
  while (hi - lo > 1) {
    long long mid = lo + (hi - lo) / 2;
    if (enc_u(mid, c, nvbin) >= thr)
      hi = mid;
    else
      lo = mid;
  }
  bnd[n] = hi;
}

// rt[v+half] = the code a zero kick gives code v: decode, then encode with the
// same sigma (the reference's FP64 expressions, update_particle.f90:67,117);
// a particle whose PP force is zero takes its code from here
__global__ void k_reencode(CodecView k, const float* sigp, float sigma, int nvbin, int32_t* __restrict__ rt) {
  if (sigp) sigma = *sigp;
  k.cf = (float)vcoef(sigma);
  k.cfp = nullptr;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < nvbin) rt[i] = (int32_t)codec_encode(k, codec_decode(k, i - k.half));
}

static void view_of(const cube_ctx* c, const cube_ctx::Codec& k, CodecView* v) {
  v->dec = k.dec;
  v->dech = k.dech;
  v->bnd = k.bnd;
  v->half = c->nvbin / 2;
  v->nmax = c->nvbin / 2 - 1;
  v->cf = (float)vcoef_host(k.sigma);
  v->amp = (float)((double)(c->nvbin - 1) / (double)CUBE_PI_F);
  v->cfp = nullptr;
  v->rt = k.rt;
}

static int build_codec(cube_ctx* c, int slot, float sigma, const float* sigp = nullptr) {
  cube_ctx::Codec& k = c->codec[slot];
  k_decode_table<<<(c->nvbin + 255) / 256, 256, 0, c->stream>>>(c->tan_tab, c->nvbin, sigma, sigp, k.dec, k.dech);
  int nmax = c->nvbin / 2 - 1;
  k_encode_bounds<<<(nmax + 127) / 128, 128, 0, c->stream>>>(sigma, sigp, c->nvbin, k.bnd);
  if (k.rt) {
    CodecView v;
    view_of(c, k, &v);
    k_reencode<<<(c->nvbin + 255) / 256, 256, 0, c->stream>>>(v, sigp, sigma, c->nvbin, k.rt);
  }
  CUBE_CUDA(c, cudaGetLastError());
  k.sigma = sigma;
  return CUBE_OK;
}

// graph mode: the tables of slot from the sigma in device memory, and a view
// of a slot whose estimate coefficient is read from the device
int cube_codec_build_dev(cube_ctx* c, int slot, const float* sigp) { return build_codec(c, slot, -1.f, sigp); }
void cube_codec_view_dev(const cube_ctx* c, int slot, const float* cfp, CodecView* v) {
  view_of(c, c->codec[slot], v);
  v->cf = 0.f;
  v->cfp = cfp;
}

// Make the tables for s1 and s2 resident (at most two slots; the slot of the
// other requested sigma is never evicted).
int cube_codec_pair(cube_ctx* c, float s1, float s2, CodecView* v1, CodecView* v2) {
  if (!(s1 > 0.f) || !(s2 > 0.f)) return cube_fail(c, CUBE_ERR_ARG, "sigma_vi must be positive");
  int i1 = c->codec[0].sigma == s1 ? 0 : (c->codec[1].sigma == s1 ? 1 : -1);
  int i2 = c->codec[0].sigma == s2 ? 0 : (c->codec[1].sigma == s2 ? 1 : -1);
  if (i1 < 0) {
    i1 = (i2 >= 0) ? 1 - i2 : c->codec_next;
    int r = build_codec(c, i1, s1);
    if (r) return r;
    c->codec_next = 1 - i1;
  }
  if (i2 < 0) {
    i2 = (s2 == s1) ? i1 : 1 - i1;
    if (i2 != i1) {
      int r = build_codec(c, i2, s2);
      if (r) return r;
      c->codec_next = 1 - i2;
    }
  }
  if (v1) view_of(c, c->codec[i1], v1);
  if (v2) view_of(c, c->codec[i2], v2);
  return CUBE_OK;
}

int cube_stats_fetch(cube_ctx* c) {
  CUBE_CUDA(c, cudaMemcpyAsync(c->hstats, c->dstats, sizeof(DevStats), cudaMemcpyDeviceToHost, c->stream));
  CUBE_CUDA(c, cudaStreamSynchronize(c->stream));
  return CUBE_OK;
}

// ------------------------------------------------------ codec self check
__global__ void k_codec_check(const double* __restrict__ v, int64_t n, double c, int nvbin, CodecView k,
                              int32_t* __restrict__ direct, int32_t* __restrict__ table) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    direct[i] = (int32_t)v_encode(v[i], c, nvbin);
    int32_t t = (int32_t)codec_encode(k, v[i]);
    // the kernels' certified encode (its table-free test first): when it
    // certifies a code, that code must be the table's; INT32_MIN marks a miss
    const long long bits = __double_as_longlong(v[i]);
    long long nq;
    if (certify_abs(bits & 0x7fffffffffffffffLL, 0.f, k, &nq) && (bits < 0 ? -nq : nq) != (long long)t) t = INT32_MIN;
    table[i] = t;
  }
}

extern "C" int cube_codec_check(cube_ctx* c, float sigma, const double* v, int64_t n, int32_t* direct,
                                int32_t* table) {
  if (!c || !v || !direct || !table || n < 0) return CUBE_ERR_ARG;
  CUBE_CUDA(c, cudaSetDevice(c->device));
  CodecView k;
  int r = cube_codec_pair(c, sigma, sigma, &k, nullptr);
  if (r) return r;
  double* dv = nullptr;
  int32_t *dd = nullptr, *dt = nullptr;
  CUBE_CUDA(c, cudaMalloc(&dv, 8 * (size_t)n + 8));
  CUBE_CUDA(c, cudaMalloc(&dd, 4 * (size_t)n + 4));
  CUBE_CUDA(c, cudaMalloc(&dt, 4 * (size_t)n + 4));
  CUBE_CUDA(c, cudaMemcpyAsync(dv, v, 8 * (size_t)n, cudaMemcpyHostToDevice, c->stream));
  k_codec_check<<<cube_grid(n, 256), 256, 0, c->stream>>>(dv, n, vcoef_host(sigma), c->nvbin, k, dd, dt);
  CUBE_CUDA(c, cudaGetLastError());
  CUBE_CUDA(c, cudaMemcpyAsync(direct, dd, 4 * (size_t)n, cudaMemcpyDeviceToHost, c->stream));
  CUBE_CUDA(c, cudaMemcpyAsync(table, dt, 4 * (size_t)n, cudaMemcpyDeviceToHost, c->stream));
  CUBE_CUDA(c, cudaStreamSynchronize(c->stream));
  cudaFree(dv);
  cudaFree(dd);
  cudaFree(dt);
  return CUBE_OK;
}

// ------------------------------------------------------ arithmetic self check
// Every float bit pattern x (NaN excluded): div_const(x, c, RN(1/c)) against
// the IEEE division __fdiv_rn(x, c) for c = 6 and c = pi_f, the two divisors of
// the kick terms.  Counts differing results (bitwise) per divisor.
__global__ void k_arith_check(unsigned long long* mism) {
  unsigned long long m6 = 0, mpi = 0;
  const float r6 = __frcp_rn(6.0f), rpi = __frcp_rn(CUBE_PI_F);
  for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < (1ull << 32);
       i += (unsigned long long)gridDim.x * blockDim.x) {
    float x = __uint_as_float((unsigned int)i);
    if (x != x) continue;
    m6 += __float_as_uint(div_const(x, 6.0f, r6)) != __float_as_uint(__fdiv_rn(x, 6.0f));
    mpi += __float_as_uint(div_const(x, CUBE_PI_F, rpi)) != __float_as_uint(__fdiv_rn(x, CUBE_PI_F));
  }
  for (int o = 16; o > 0; o >>= 1) {
    m6 += __shfl_xor_sync(0xffffffffu, m6, o);
    mpi += __shfl_xor_sync(0xffffffffu, mpi, o);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(mism, m6);
    atomicAdd(mism + 1, mpi);
  }
}

extern "C" int cube_arith_check(cube_ctx* c, int64_t* mismatches) {
  if (!c || !mismatches) return CUBE_ERR_ARG;
  CUBE_CUDA(c, cudaSetDevice(c->device));
  unsigned long long* d = reinterpret_cast<unsigned long long*>(c->red_tmp);  // >= 2 doubles of scratch
  CUBE_CUDA(c, cudaMemsetAsync(d, 0, 2 * sizeof(unsigned long long), c->stream));
  k_arith_check<<<cube_grid((int64_t)1 << 32, 256, 8), 256, 0, c->stream>>>(d);
  CUBE_CUDA(c, cudaGetLastError());
  unsigned long long h[2] = {0, 0};
  CUBE_CUDA(c, cudaMemcpyAsync(h, d, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
  CUBE_CUDA(c, cudaStreamSynchronize(c->stream));
  mismatches[0] = (int64_t)h[0];
  mismatches[1] = (int64_t)h[1];
  return CUBE_OK;
}

// ------------------------------------------------- codec check, static scratch
// cube_codec_check_static: the same check with all of its device scratch in a
// file-scope array instead of per-call cudaMalloc/cudaFree.  It serves callers
// that must not allocate device memory: a production run sizes np_max to fill
// most of HBM, so a mid-run cudaMalloc can fail or fragment the pool, and
// cudaFree synchronises the whole device, which stalls every other stream.
// The array holds CUBE_CODEC_STATIC_MAX doubles of input, two
// CUBE_CODEC_STATIC_MAX int32 outputs and one set of codec tables for the
// largest velocity format (izipv = 2: 65536 decode values as double and as a
// float pair, 32769 encode bounds), 1.25 MiB + 256 KiB in all.  The tables
// are rebuilt by every call for its sigma, so the context's own two codec
// slots (the step's sigma_vi and sigma_vi_new) are never touched.  Nothing in
// the array needs to start at zero: each call writes every value it reads.
// All contexts on one device share the array, so two calls whose device work
// overlapped would race; each call holds a per-device host lock from its
// first launch until its stream has drained.
constexpr int64_t kStaticNvbin = 65536;  // 2^(8*izipv) for izipv <= 2
constexpr int64_t kStaticIoBytes = CUBE_CODEC_STATIC_MAX * (8 + 4 + 4);
constexpr int64_t kStaticTabBytes = kStaticNvbin * 8 + kStaticNvbin * 8 + (kStaticNvbin / 2 + 1) * 8;
constexpr int64_t kCodecStaticBytes = kStaticIoBytes + kStaticTabBytes;
static_assert(kStaticIoBytes % 256 == 0, "the tables start 256-byte aligned");
static __device__ __align__(256) unsigned char g_codec_scratch[kCodecStaticBytes];

namespace {
constexpr int kMaxDevices = 64;
std::mutex g_codec_scratch_mu[kMaxDevices];
unsigned char* g_codec_scratch_ptr[kMaxDevices] = {};  // device address, per device
}  // namespace

// First call on a device (with that device current) resolves the array's
// device address; that resolution may load this module's device code, so the
// first call belongs before any stream capture.
static int codec_scratch_address(cube_ctx* c, unsigned char** out) {
  if (!g_codec_scratch_ptr[c->device]) {
    void* ptr = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&ptr, g_codec_scratch);
    if (e != cudaSuccess || !ptr)
      return cube_fail(c, CUBE_ERR_CUDA, std::string("cudaGetSymbolAddress(codec scratch): ") + cudaGetErrorString(e));
    g_codec_scratch_ptr[c->device] = static_cast<unsigned char*>(ptr);
  }
  *out = g_codec_scratch_ptr[c->device];
  return CUBE_OK;
}

extern "C" int cube_codec_check_static(cube_ctx* c, float sigma, const double* v, int64_t n, int32_t* direct,
                                       int32_t* table) {
  if (!c || !v || !direct || !table || n < 0) return CUBE_ERR_ARG;
  if (n > CUBE_CODEC_STATIC_MAX)
    return cube_fail(c, CUBE_ERR_ARG, "n = " + std::to_string(n) + " exceeds the static scratch maximum of " +
                                          std::to_string((long long)CUBE_CODEC_STATIC_MAX) + " values");
  if (!(sigma > 0.f)) return cube_fail(c, CUBE_ERR_ARG, "sigma_vi must be positive");
  if (c->device < 0 || c->device >= kMaxDevices) return cube_fail(c, CUBE_ERR_ARG, "device ordinal out of range");
  if (c->nvbin > kStaticNvbin) return cube_fail(c, CUBE_ERR_ARG, "velocity format wider than the static tables");
  CUBE_CUDA(c, cudaSetDevice(c->device));
  std::lock_guard<std::mutex> lock(g_codec_scratch_mu[c->device]);
  unsigned char* base = nullptr;
  int r = codec_scratch_address(c, &base);
  if (r) return r;
  if (n == 0) return CUBE_OK;
  double* dv = reinterpret_cast<double*>(base);
  int32_t* dd = reinterpret_cast<int32_t*>(base + 8 * CUBE_CODEC_STATIC_MAX);
  int32_t* dt = reinterpret_cast<int32_t*>(base + 12 * CUBE_CODEC_STATIC_MAX);
  cube_ctx::Codec tab;
  tab.sigma = sigma;
  tab.dec = reinterpret_cast<double*>(base + kStaticIoBytes);
  tab.dech = reinterpret_cast<float2*>(base + kStaticIoBytes + 8 * kStaticNvbin);
  tab.bnd = reinterpret_cast<long long*>(base + kStaticIoBytes + 16 * kStaticNvbin);
  CodecView k;
  view_of(c, tab, &k);
  // every early return below first drains the stream, so the lock is never
  // released with work on the shared array still in flight
  const int nmax = c->nvbin / 2 - 1;
  k_decode_table<<<(c->nvbin + 255) / 256, 256, 0, c->stream>>>(c->tan_tab, c->nvbin, sigma, nullptr, tab.dec,
                                                                  tab.dech);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) {
    k_encode_bounds<<<(nmax + 127) / 128, 128, 0, c->stream>>>(sigma, nullptr, c->nvbin, tab.bnd);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(dv, v, 8 * (size_t)n, cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess) {
    k_codec_check<<<cube_grid(n, 256), 256, 0, c->stream>>>(dv, n, vcoef_host(sigma), c->nvbin, k, dd, dt);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(direct, dd, 4 * (size_t)n, cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(table, dt, 4 * (size_t)n, cudaMemcpyDeviceToHost, c->stream);
  cudaError_t es = cudaStreamSynchronize(c->stream);
  if (e == cudaSuccess) e = es;
  if (e != cudaSuccess) return cube_fail(c, CUBE_ERR_CUDA, std::string("codec check (static scratch): ") + cudaGetErrorString(e));
  return CUBE_OK;
}
