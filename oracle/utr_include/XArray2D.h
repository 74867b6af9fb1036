/* XArray2D.h (shim) -- a dense [dim1][dim2] array (dim2 fastest).  See
 * XA_ini.h.  TEST INFRASTRUCTURE ONLY. */
#pragma once
#include "XA_ini.h"

namespace xar {
template <class T> class XArray2D {
public:
    XArray2D(index_t n1 = 0, index_t n2 = 0) : n1_(n1), n2_(n2), d_(n1 * n2) {}
    index_t GetDim1() const { return n1_; }
    index_t GetDim2() const { return n2_; }
    T *operator[](index_t j) { return d_.data() + j * n2_; }
    const T *operator[](index_t j) const { return d_.data() + j * n2_; }
    T *data() { return d_.data(); }

private:
    index_t n1_, n2_;
    std::vector<T> d_;
};
}  // namespace xar
