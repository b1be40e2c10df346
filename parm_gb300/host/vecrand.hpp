// parm_gb300 host API: vectors, scalar types and random numbers with the
// names of the reference's src/vecrand.hpp (wackywendell/parm), so that code
// written against the reference compiles unchanged against this library.
//
// Build for 3D (default, -DVEC3D) or 2D (-DVEC2D), as the reference.  Vec is a
// fixed-size vector with the subset of Eigen's interface that the MD path
// uses; its reductions evaluate in the order Eigen's fixed-size 2- and 3-
// vectors use ((v0 op v1) op v2), the order the GPU path reproduces.
#ifndef PARM_GB300_VECRAND_HPP
#define PARM_GB300_VECRAND_HPP

#ifdef VEC2D
#define NDIM 2
#else
#ifndef VEC3D
#define VEC3D
#endif
#define NDIM 3
#endif

#include <cmath>
#include <ctime>
#include <iostream>
#include <memory>
#include <random>
#include <stdexcept>
#include <vector>

using namespace std;

typedef unsigned int uint;
typedef const unsigned int cuint;
typedef double flt;

const flt OVERNDIM = ((flt)1.0) / NDIM;

// shared pointers: the reference uses boost::shared_ptr through `sptr`
template <class T>
using sptr = std::shared_ptr<T>;
namespace boost {
using std::dynamic_pointer_cast;
using std::shared_ptr;
using std::static_pointer_cast;
}  // namespace boost

//! Fixed-size FP64 vector (the reference's Eigen::Matrix<flt, N, 1>).
template <int N>
struct VecN {
    flt c[N];

    VecN() {
        for (int d = 0; d < N; d++) c[d] = 0;
    }
    VecN(flt x, flt y) {
        static_assert(N == 2, "two coefficients for a 2-vector");
        c[0] = x;
        c[1] = y;
    }
    VecN(flt x, flt y, flt z) {
        static_assert(N == 3, "three coefficients for a 3-vector");
        c[0] = x;
        c[1] = y;
        c[2] = z;
    }
    static VecN Zero() { return VecN(); }
    static VecN Ones() {
        VecN v;
        for (int d = 0; d < N; d++) v.c[d] = 1;
        return v;
    }
    static int size() { return N; }
    flt& operator[](int i) { return c[i]; }
    const flt& operator[](int i) const { return c[i]; }
    flt& operator()(int i) { return c[i]; }
    const flt& operator()(int i) const { return c[i]; }
    flt* data() { return c; }
    const flt* data() const { return c; }
    void setZero() {
        for (int d = 0; d < N; d++) c[d] = 0;
    }

    VecN operator+(const VecN& o) const {
        VecN r;
        for (int d = 0; d < N; d++) r.c[d] = c[d] + o.c[d];
        return r;
    }
    VecN operator-(const VecN& o) const {
        VecN r;
        for (int d = 0; d < N; d++) r.c[d] = c[d] - o.c[d];
        return r;
    }
    VecN operator-() const {
        VecN r;
        for (int d = 0; d < N; d++) r.c[d] = -c[d];
        return r;
    }
    VecN operator*(flt s) const {
        VecN r;
        for (int d = 0; d < N; d++) r.c[d] = c[d] * s;
        return r;
    }
    VecN operator/(flt s) const {
        VecN r;
        for (int d = 0; d < N; d++) r.c[d] = c[d] / s;
        return r;
    }
    VecN& operator+=(const VecN& o) {
        for (int d = 0; d < N; d++) c[d] += o.c[d];
        return *this;
    }
    VecN& operator-=(const VecN& o) {
        for (int d = 0; d < N; d++) c[d] -= o.c[d];
        return *this;
    }
    VecN& operator*=(flt s) {
        for (int d = 0; d < N; d++) c[d] *= s;
        return *this;
    }
    VecN& operator/=(flt s) {
        for (int d = 0; d < N; d++) c[d] /= s;
        return *this;
    }
    bool operator==(const VecN& o) const {
        for (int d = 0; d < N; d++)
            if (c[d] != o.c[d]) return false;
        return true;
    }
    bool operator!=(const VecN& o) const { return !(*this == o); }

    flt dot(const VecN& o) const {
        flt s = c[0] * o.c[0];
        for (int d = 1; d < N; d++) s = s + c[d] * o.c[d];
        return s;
    }
    flt squaredNorm() const { return dot(*this); }
    flt norm() const { return std::sqrt(squaredNorm()); }
    VecN normalized() const { return *this / norm(); }
    flt sum() const {
        flt s = c[0];
        for (int d = 1; d < N; d++) s = s + c[d];
        return s;
    }
    flt prod() const {
        flt s = c[0];
        for (int d = 1; d < N; d++) s = s * c[d];
        return s;
    }
    VecN cwiseProduct(const VecN& o) const {
        VecN r;
        for (int d = 0; d < N; d++) r.c[d] = c[d] * o.c[d];
        return r;
    }
    VecN cwiseQuotient(const VecN& o) const {
        VecN r;
        for (int d = 0; d < N; d++) r.c[d] = c[d] / o.c[d];
        return r;
    }
};

template <int N>
inline VecN<N> operator*(flt s, const VecN<N>& v) {
    return v * s;
}

template <int N>
inline std::ostream& operator<<(std::ostream& os, const VecN<N>& v) {
    for (int d = 0; d < N; d++) os << (d ? " " : "") << v.c[d];
    return os;
}

typedef VecN<NDIM> Vec;
typedef VecN<2> Vec2;
typedef VecN<3> Vec3;

//! NDIM x NDIM matrix (stress tensors), row-major coefficients.
struct Matrix {
    flt c[NDIM][NDIM];
    Matrix() {
        for (int a = 0; a < NDIM; a++)
            for (int b = 0; b < NDIM; b++) c[a][b] = 0;
    }
    static Matrix Zero() { return Matrix(); }
    flt& operator()(int a, int b) { return c[a][b]; }
    const flt& operator()(int a, int b) const { return c[a][b]; }
};

//! Rows of NDIM values (the reference's Eigen::Matrix<flt, Eigen::Dynamic,
//! NDIM>: rows(), cols(), row(i), (i, d), size()).
struct VecRows {
    std::vector<Vec> r;
    VecRows() {}
    explicit VecRows(size_t n) : r(n, Vec::Zero()) {}
    size_t rows() const { return r.size(); }
    static constexpr size_t cols() { return NDIM; }
    size_t size() const { return r.size() * NDIM; }
    Vec row(size_t i) const { return r[i]; }
    flt& operator()(size_t i, size_t d) { return r[i][d]; }
    flt operator()(size_t i, size_t d) const { return r[i][d]; }
};

#ifdef VEC3D
inline Vec vec() { return Vec(0, 0, 0); }
#else
inline Vec vec() { return Vec(0, 0); }
#endif

// Random numbers.  The reference draws from Boost's mt19937; this library
// uses std::mt19937 with the same seeding interface (streams differ).
std::mt19937& parm_random_engine();
flt rand01();
Vec rand_vec();
Vec rand_vec_boxed();
unsigned int seed(unsigned int n);
unsigned int seed();

#endif
