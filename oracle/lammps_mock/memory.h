/* LAMMPS-style memory helpers (TEST INFRASTRUCTURE ONLY): 1-D arrays and 2-D
 * arrays stored contiguously with a row-pointer table, grown in place with
 * their old contents kept, as the engine's Memory::grow does. */
#ifndef EPH_MOCK_MEMORY_H
#define EPH_MOCK_MEMORY_H
#include "lammps.h"
#include <cstdlib>

namespace LAMMPS_NS {
class Memory {
 public:
  template <typename T> T *grow(T *&a, int n, const char *) {
    T *p = static_cast<T *>(std::realloc(a, sizeof(T) * (n > 0 ? n : 1)));
    if (!p) throw std::bad_alloc();
    a = p;
    return a;
  }
  template <typename T> T **grow(T **&a, int n1, int n2, const char *) {
    T *data = a ? a[0] : nullptr;
    data = static_cast<T *>(std::realloc(data, sizeof(T) * (size_t)(n1 > 0 ? n1 : 1) * n2));
    T **rows = static_cast<T **>(std::realloc(a, sizeof(T *) * (n1 > 0 ? n1 : 1)));
    if (!data || !rows) throw std::bad_alloc();
    for (int i = 0; i < n1; ++i) rows[i] = data + (size_t)i * n2;
    a = rows;
    return a;
  }
  template <typename T> void destroy(T *&a) { std::free(a); a = nullptr; }
  template <typename T> void destroy(T **&a) {
    if (a) std::free(a[0]);
    std::free(a);
    a = nullptr;
  }
};
}  // namespace LAMMPS_NS
#endif
