/*
 * Fixed-size vectors for case hook code: the operations the plug-in surface
 * uses on `vect` (component access, element-wise arithmetic with vectors and
 * scalars, scalar fill `v = 0.0`, comma lists `v = 1, 2, 3;`, len / len2 /
 * dot), sized by the case's NDIM.
 */
#ifndef SPHDEM_FACADE_VECT_H
#define SPHDEM_FACADE_VECT_H

#include <cmath>
#include <iomanip>
#include <ostream>

#include "customConstants.h"

template <typename T, int N>
class TVect {
   public:
    T x[N];

    TVect() {
        for (int i = 0; i < N; i++) x[i] = T(0);
    }
    TVect(T a) {  // `vect v = 0.0;`
        for (int i = 0; i < N; i++) x[i] = a;
    }
    TVect(T a, T b) {
        const T v[2] = {a, b};
        for (int i = 0; i < N; i++) x[i] = i < 2 ? v[i] : T(0);
    }
    TVect(T a, T b, T c) {
        const T v[3] = {a, b, c};
        for (int i = 0; i < N; i++) x[i] = i < 3 ? v[i] : T(0);
    }
    /* `vect v = ARRAY;` from a case constant such as RMIN[NDIM] */
    TVect(const T (&a)[N]) {
        for (int i = 0; i < N; i++) x[i] = a[i];
    }
    T &operator[](int i) { return x[i]; }
    const T &operator[](int i) const { return x[i]; }

    /* `v = s` fills every component; `v = a, b, c` sets them in turn */
    class Lister {
       public:
        Lister(TVect &v, int next) : v_(v), next_(next) {}
        Lister operator,(T a) {
            if (next_ < N) v_.x[next_] = a;
            return Lister(v_, next_ + 1);
        }

       private:
        TVect &v_;
        int next_;
    };
    Lister operator=(T a) {
        for (int i = 0; i < N; i++) x[i] = a;
        return Lister(*this, 1);
    }
    TVect &operator=(const TVect &o) = default;
    TVect(const TVect &o) = default;

    TVect &operator+=(const TVect &o) {
        for (int i = 0; i < N; i++) x[i] += o.x[i];
        return *this;
    }
    TVect &operator-=(const TVect &o) {
        for (int i = 0; i < N; i++) x[i] -= o.x[i];
        return *this;
    }
    TVect &operator*=(T a) {
        for (int i = 0; i < N; i++) x[i] *= a;
        return *this;
    }
    TVect &operator/=(T a) {
        for (int i = 0; i < N; i++) x[i] /= a;
        return *this;
    }
};

template <typename T, int N>
inline TVect<T, N> operator+(TVect<T, N> a, const TVect<T, N> &b) { return a += b; }
template <typename T, int N>
inline TVect<T, N> operator-(TVect<T, N> a, const TVect<T, N> &b) { return a -= b; }
template <typename T, int N>
inline TVect<T, N> operator-(TVect<T, N> a) {
    for (int i = 0; i < N; i++) a.x[i] = -a.x[i];
    return a;
}
template <typename T, int N>
inline TVect<T, N> operator*(T s, TVect<T, N> a) { return a *= s; }
template <typename T, int N>
inline TVect<T, N> operator*(TVect<T, N> a, T s) { return a *= s; }
template <typename T, int N>
inline TVect<T, N> operator/(TVect<T, N> a, T s) { return a /= s; }

template <typename T, int N>
inline T dot(const TVect<T, N> &a, const TVect<T, N> &b) {
    T s = T(0);
    for (int i = 0; i < N; i++) s += a.x[i] * b.x[i];
    return s;
}
template <typename T, int N>
inline T len2(const TVect<T, N> &a) { return dot(a, a); }
template <typename T, int N>
inline T len(const TVect<T, N> &a) { return std::sqrt(len2(a)); }

/* element-wise product and quotient, as blitz's TinyVector arithmetic */
template <typename T, int N>
inline TVect<T, N> operator*(TVect<T, N> a, const TVect<T, N> &b) {
    for (int i = 0; i < N; i++) a.x[i] *= b.x[i];
    return a;
}
template <typename T, int N>
inline TVect<T, N> operator/(TVect<T, N> a, const TVect<T, N> &b) {
    for (int i = 0; i < N; i++) a.x[i] /= b.x[i];
    return a;
}

/* the text blitz writes for a TinyVector (its tinyvecio.cc layout): the
 * length, then the components in fields of width 10 between brackets, a line
 * break after every seventh */
template <typename T, int N>
inline std::ostream &operator<<(std::ostream &os, const TVect<T, N> &a) {
    os << N << " [ ";
    for (int i = 0; i < N; i++) {
        os << std::setw(10) << a.x[i];
        if ((i + 1) % 7 == 0) os << std::endl << "  ";
    }
    os << " ]";
    return os;
}

typedef TVect<double, NDIM> vect;
typedef TVect<int, NDIM> vectInt;

#endif
