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
}  // namespace hss
