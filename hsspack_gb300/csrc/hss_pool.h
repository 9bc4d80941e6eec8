// hss_pool.h -- named grow-only device buffers owned by the library context.
#pragma once
#include <cstddef>

namespace hss {
// Device buffer `name` of at least `bytes` (contents persist between calls
// until the buffer grows).  Throws on allocation failure.
void *pool_get(const char *name, size_t bytes);
template <class T>
inline T *pool(const char *name, size_t count) {
  return (T *)pool_get(name, count * sizeof(T));
}
// Host -> device copy of a parameter array (asynchronous on `stream`; the
// source may be reused at once): pageable when small, through a pinned
// staging ring when large.
void stage_h2d(void *dst, const void *src, size_t bytes, void *stream);
// Stage timing hooks (active when hss_config.profile = 1): begin/end record
// CUDA events on `st`; bytes/flops are the stage's algorithmic work.
void stage_begin(int stage, void *st);
void stage_end(int stage, void *st, long long bytes, double flops);
}  // namespace hss
