// Radix sort of (key, entry) pairs for the re-sort's general rank path
// (cube_update.cu): CUB's stable LSD DeviceRadixSort over a bit range of
// 64-bit keys.  A translation unit of its own: the sort's templates are the
// slowest part of the build.
#include <climits>
#include <cub/device/device_radix_sort.cuh>

#include "cube_internal.cuh"

int cube_sort_pairs(cube_ctx* c, int64_t n, int begin_bit, int end_bit, uint64_t** keys, int32_t** vals) {
  const int64_t cap = c->p.np_max + c->xtra_cap;
  if (n > cap || cap >= INT_MAX) return cube_fail(c, CUBE_ERR_ARG, "sort: too many entries");
  if (!c->skey[0]) {  // first use: both buffers of keys and entries, 24 bytes an entry
    for (int i = 0; i < 2; i++) {
      if (cudaMalloc(&c->skey[i], 8 * (size_t)cap) != cudaSuccess ||
          cudaMalloc(&c->sval[i], 4 * (size_t)cap) != cudaSuccess)
        return cube_fail(c, CUBE_ERR_NOMEM, "re-sort keys");
    }
  }
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
