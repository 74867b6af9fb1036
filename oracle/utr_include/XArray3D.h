/* XArray3D.h (shim) -- a dense [dim1][dim2][dim3] array (dim3 fastest).  See
 * XA_ini.h.  TEST INFRASTRUCTURE ONLY. */
#pragma once
#include "XA_ini.h"

namespace xar {
template <class T> class XArray3D {
public:
    struct Plane {
        T *p;
        index_t n3;
        T *operator[](index_t j) const { return p + j * n3; }
    };
    XArray3D(index_t n1 = 0, index_t n2 = 0, index_t n3 = 0)
        : n1_(n1), n2_(n2), n3_(n3), d_(n1 * n2 * n3) {}
    index_t GetDim1() const { return n1_; }
    index_t GetDim2() const { return n2_; }
    index_t GetDim3() const { return n3_; }
    Plane operator[](index_t k) { return Plane{d_.data() + k * n2_ * n3_, n3_}; }
    T *data() { return d_.data(); }

private:
    index_t n1_, n2_, n3_;
    std::vector<T> d_;
};
}  // namespace xar
