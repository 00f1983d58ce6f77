/* HEALPix C++ compatibility shim (TEST INFRASTRUCTURE ONLY): rangeset. */
#ifndef PISCO_SHIM_RANGESET_H
#define PISCO_SHIM_RANGESET_H
#include <vector>
template <typename T> class rangeset {
    std::vector<T> r;
  public:
    void clear() { r.clear(); }
    void append(T a, T b) {
        if (b <= a) return;
        if (!r.empty() && a <= r.back()) {
            if (b > r.back()) r.back() = b;
        } else {
            r.push_back(a);
            r.push_back(b);
        }
    }
    std::size_t nranges() const { return r.size() / 2; }
    const T& ivbegin(std::size_t i) const { return r[2 * i]; }
    const T& ivend(std::size_t i) const { return r[2 * i + 1]; }
};
#endif
