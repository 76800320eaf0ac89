// Chunking of the host-buffer imaging path (litho_image_batch with host
// pointers): how many masks one chunk carries and the order of chunk sizes.
// Plain C++ with no CUDA, so the schedule is also checked on the CPU.
#pragma once
#include <algorithm>
#include <cstddef>
#include <vector>

namespace litho {

// Masks per chunk: up to chunk_bytes of masks and at least ~8 chunks, so small batches
// pipeline too; never below one mask.  The host link moves chunked copies in both
// directions at once faster the larger the chunk (GB300 to Grace memory, pinned: 314 GB/s
// at 16 MB, 333 at 64 MB, 338 at 128 MB, 340 at 256 MB), against three staging slots of
// that size per direction on the device.
constexpr size_t HOST_CHUNK_BYTES = (size_t)128 << 20;

inline int host_chunk_masks(int batch, size_t img_bytes, size_t chunk_bytes = HOST_CHUNK_BYTES) {
  const size_t cap = std::min<size_t>(chunk_bytes / img_bytes, ((size_t)batch + 7) / 8);
  return (int)std::max<size_t>(1, cap);
}

// chunk sizes: a ramp 1, 2, 4, ... (each below CH) at the start, CH-sized chunks
// (the last of them ragged) in the middle and the ramp reversed at the end, so
// the first copy in and the last copy out, which nothing overlaps, are short.  A
// ramp step is taken only while at least one full CH chunk stays in the middle.
inline void chunk_schedule(int batch, int CH, std::vector<int>& sizes) {
  std::vector<int> ramp;
  int used = 0;
  for (int r = 1; r < CH && 2 * (used + r) + CH <= batch; r *= 2) {
    ramp.push_back(r);
    used += r;
  }
  sizes.assign(ramp.begin(), ramp.end());
  for (int mid = batch - 2 * used; mid > 0; mid -= CH) sizes.push_back(std::min(CH, mid));
  sizes.insert(sizes.end(), ramp.rbegin(), ramp.rend());
}

}  // namespace litho
