// Radix sort of (key, entry) pairs for the re-sort's general rank path
// (cube_update.cu): CUB's stable LSD DeviceRadixSort over a bit range of
// 64-bit keys.  A translation unit of its own: the sort's templates are the
// slowest part of the build.
#include <climits>
#include <cub/device/device_radix_sort.cuh>

#include "cube_internal.cuh"

// One device allocation of the sort buffers; the fault-injection option
// (CUBE_OPT_FAIL_ALLOC) makes the n-th such allocation report failure.
static cudaError_t sort_alloc(cube_ctx* c, void** p, size_t bytes) {
  if (c->fail_alloc > 0 && --c->fail_alloc == 0) return cudaErrorMemoryAllocation;
  return cudaMalloc(p, bytes);
}

// Both buffers of keys and entries (24 bytes an entry), all four or none: a
// failure frees what was made, so the next call tries again instead of
// sorting into a missing buffer.
static int sort_buffers(cube_ctx* c, int64_t cap) {
  if (c->skey[0] && c->skey[1] && c->sval[0] && c->sval[1]) return CUBE_OK;
  void* p[4] = {nullptr, nullptr, nullptr, nullptr};
  const size_t bytes[4] = {8 * (size_t)cap, 8 * (size_t)cap, 4 * (size_t)cap, 4 * (size_t)cap};
  for (int i = 0; i < 4; i++) {
    if (sort_alloc(c, &p[i], bytes[i]) != cudaSuccess) {
      cudaGetLastError();  // a failed cudaMalloc is also the thread's last error: clear it
      for (int j = 0; j < i; j++) cudaFree(p[j]);
      return cube_fail(c, CUBE_ERR_NOMEM, "re-sort keys: cudaMalloc of " + std::to_string(bytes[i]) + " bytes failed");
    }
  }
  c->skey[0] = static_cast<uint64_t*>(p[0]);
  c->skey[1] = static_cast<uint64_t*>(p[1]);
  c->sval[0] = static_cast<int32_t*>(p[2]);
  c->sval[1] = static_cast<int32_t*>(p[3]);
  return CUBE_OK;
}

int cube_sort_pairs(cube_ctx* c, int64_t n, int begin_bit, int end_bit, uint64_t** keys, int32_t** vals) {
  const int64_t cap = c->p.np_max + c->xtra_cap;
  if (n > cap || cap >= INT_MAX) return cube_fail(c, CUBE_ERR_ARG, "sort: too many entries");
  int r = sort_buffers(c, cap);
  if (r) return r;
  *keys = c->skey[0];
  *vals = c->sval[0];
  if (n == 0) return CUBE_OK;
  cub::DoubleBuffer<uint64_t> dk(c->skey[0], c->skey[1]);
  cub::DoubleBuffer<int32_t> dv(c->sval[0], c->sval[1]);
  size_t bytes = 0;
  CUBE_CUDA(c, cub::DeviceRadixSort::SortPairs(nullptr, bytes, dk, dv, (int)n, begin_bit, end_bit, c->stream));
  if (bytes > c->sort_tmp_bytes) {
    if (c->sort_tmp) cudaFree(c->sort_tmp);
    c->sort_tmp = nullptr;
    c->sort_tmp_bytes = 0;
    if (cudaMalloc(&c->sort_tmp, bytes) != cudaSuccess) return cube_fail(c, CUBE_ERR_NOMEM, "re-sort scratch");
    c->sort_tmp_bytes = bytes;
  }
  CUBE_CUDA(c, cub::DeviceRadixSort::SortPairs(c->sort_tmp, bytes, dk, dv, (int)n, begin_bit, end_bit, c->stream));
  *keys = dk.Current();
  *vals = dv.Current();
  return CUBE_OK;
}
