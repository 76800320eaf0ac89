// Chunking of the host-buffer imaging path (litho_image_batch with host
// pointers): how many masks one chunk carries and the order of chunk sizes.
// Plain C++ with no CUDA, so the schedule is also checked on the CPU.
#pragma once
#include <algorithm>
#include <cstddef>
#include <vector>

namespace litho {

// masks per chunk: up to ~16 MB of masks (enough per launch in the steady state)
// and at least ~8 chunks, so small images pipeline too; never below one mask
inline int host_chunk_masks(int batch, size_t img_bytes) {
  const size_t cap = std::min<size_t>(((size_t)16 << 20) / img_bytes, ((size_t)batch + 7) / 8);
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
