/* HEALPix C++ compatibility shim (TEST INFRASTRUCTURE ONLY): fix_arr. */
#ifndef PISCO_SHIM_ARR_H
#define PISCO_SHIM_ARR_H
#include <cstddef>
template <typename T, std::size_t N> class fix_arr {
    T d[N];
  public:
    T& operator[](std::size_t i) { return d[i]; }
    const T& operator[](std::size_t i) const { return d[i]; }
    std::size_t size() const { return N; }
};
#endif
