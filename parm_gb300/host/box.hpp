// parm_gb300 host API: boxes and atom storage with the names of the
// reference's src/box.hpp (wackywendell/parm).
//
// AtomVec keeps the Atom records in host memory exactly as the reference
// does ({x, v, a, f, m}, 13 doubles in 3D), so caller code reads and writes
// atoms[i].x between steps as before; the GPU-backed objects (NeighborList,
// NListed, the Collections) upload these records before every GPU operation
// and download them afterwards.
#ifndef PARM_GB300_BOX_HPP
#define PARM_GB300_BOX_HPP

#include <cassert>
#include <cmath>
#include <vector>

#include "vecrand.hpp"

//! Periodic minimum image, component-wise remainder (src/box.hpp:68-78).
inline Vec vec_mod(Vec r1, const Vec r2) {
    for (int d = 0; d < NDIM; d++) r1[d] = std::remainder(r1[d], r2[d]);
    return r1;
}

class AtomGroup;

//! The shape of space and its boundaries (src/box.hpp:48-58).
class Box {
   public:
    virtual Vec diff(Vec r1, Vec r2) = 0;
    virtual flt V() = 0;
    virtual ~Box() {}
};

//! Infinite box, no boundaries (src/box.hpp:86-92).
class InfiniteBox : public Box {
   public:
    Vec diff(Vec r1, Vec r2) override { return r1 - r2; }
    flt V() override { return NAN; }
};

//! Periodic box with one corner at the origin (src/box.hpp:97-153).
class OriginBox : public Box {
   protected:
    Vec boxsize;

   public:
    explicit OriginBox(Vec size) : boxsize(size) {}
    explicit OriginBox(flt L) {
        for (int d = 0; d < NDIM; d++) boxsize[d] = L;
    }
    Vec diff(Vec r1, Vec r2) override { return vec_mod((r1 - r2), boxsize); }
    flt V() override { return boxsize.prod(); }
    flt L() { return boxsize.sum() / NDIM; }
    Vec box_shape() { return boxsize; }
    //! uniform location inside the box
    Vec rand_loc() {
        Vec v = rand_vec_boxed();
        for (int d = 0; d < NDIM; d++) v[d] *= boxsize[d];
        return diff(v, Vec::Zero());
    }
    flt resize(flt factor) {
        boxsize *= factor;
        return V();
    }
    flt resize(flt factor, AtomGroup& atoms);
    flt resize_to(Vec newsize) {
        boxsize = newsize;
        return V();
    }
    flt resize_to(Vec newsize, AtomGroup& atoms);
    flt resize_to_V(flt newV) { return resize(std::pow(newV / V(), OVERNDIM)); }
    flt resize_to_V(flt newV, AtomGroup& atoms) { return resize(std::pow(newV / V(), OVERNDIM), atoms); }
    // the current length is V^(1/NDIM), as src/box.cpp:44-55 takes it (not L())
    flt resize_to_L(flt newL) { return resize(newL / std::pow(V(), 1.0 / NDIM)); }
    flt resize_to_L(flt newL, AtomGroup& atoms) { return resize(newL / std::pow(V(), 1.0 / NDIM), atoms); }
};

//! Sheared periodic box (src/box.hpp:165-196, box.cpp:72-135): the y image
//! shifts x by gamma * Lx.  The GPU path (FP64 handles) applies the same
//! minimum image; shear(dgamma, atoms) moves the host Atom records, which
//! the next GPU call uploads.
class LeesEdwardsBox : public OriginBox {
   protected:
    flt gamma;

   public:
    LeesEdwardsBox(Vec size, flt gamma = 0.0) : OriginBox(size), gamma(gamma) {}
    LeesEdwardsBox(flt L, flt gamma = 0.0) : OriginBox(L), gamma(gamma) {}
    Vec diff(Vec r1, Vec r2) override {
        const flt Ly = boxsize[1];
        flt dy = r1[1] - r2[1];
        const int im = (int)std::round(dy / Ly);
        dy = dy - (im * Ly);
        const flt Lx = boxsize[0];
        flt dx = r1[0] - r2[0];
        dx = dx - std::round((dx / Lx) - im * gamma) * Lx - im * gamma * Lx;
        Vec r = Vec::Zero();
        r[0] = dx;
        r[1] = dy;
#ifndef VEC2D
        r[2] = std::remainder(r1[2] - r2[2], boxsize[2]);
#endif
        return r;
    }
    flt get_gamma() { return gamma; }
    void shear(flt dgamma) { gamma += dgamma; }
    void shear(flt dgamma, AtomGroup& atoms);
    void shear_to(flt new_gamma) { gamma = new_gamma; }
    void shear_to(flt new_gamma, AtomGroup& atoms);
    Vec non_affine(Vec v) {
        v[0] -= gamma * v[1];
        return v;
    }
    Vec affine(Vec v) {
        v[0] += gamma * v[1];
        return v;
    }
};

//! One particle (src/box.hpp:234-249): the layout the C ABI copies.
struct Atom {
    Vec x;
    Vec v;
    Vec a;
    Vec f;
    flt m;
};
static_assert(sizeof(Atom) == (4 * NDIM + 1) * sizeof(double), "Atom records are 4*NDIM+1 doubles");

//! An Atom together with its index in its AtomVec (src/box.hpp:257-300).
class AtomID {
   protected:
    Atom* ptr;
    uint num;

   public:
    AtomID() : ptr(nullptr), num(UINT32_MAX) {}
    AtomID(Atom* a, uint n) : ptr(a), num(n) {}
    Atom& operator*() const { return *ptr; }
    Atom* operator->() const { return ptr; }
    uint n() const { return num; }
    bool operator==(const AtomID& o) const { return ptr == o.ptr; }
    bool operator!=(const AtomID& o) const { return ptr != o.ptr; }
    bool operator<(const AtomID& o) const { return num < o.num; }
};

//! A group of atoms (src/box.hpp:330-432).
class AtomGroup {
   public:
    virtual Atom& operator[](cuint n) = 0;
    virtual Atom& operator[](cuint n) const = 0;
    virtual AtomID get_id(cuint n) = 0;
    virtual uint size() const = 0;
    Atom& get(cuint n) { return (*this)[n]; }

    flt mass() const;
    Vec momentum() const;
    Vec com_velocity() const { return momentum() / mass(); }
    flt kinetic_energy(const Vec originvelocity = Vec::Zero()) const;
    void add_velocity(Vec v);
    void reset_com_velocity() { add_velocity(-com_velocity()); }
    void reset_forces();
    void randomize_velocities(flt T);
    virtual ~AtomGroup() {}
};

//! The atoms of one simulation, in host memory (src/box.hpp:441-479).
class AtomVec : public AtomGroup {
   private:
    std::vector<Atom> atoms;

   public:
    explicit AtomVec(std::vector<double> masses) : atoms(masses.size()) {
        for (size_t i = 0; i < masses.size(); i++) atoms[i].m = masses[i];
    }
    AtomVec(uint N, flt mass) : atoms(N) {
        for (auto& a : atoms) a.m = mass;
    }
    AtomVec& vec() { return *this; }
    Atom& operator[](cuint n) override { return atoms[n]; }
    Atom& operator[](cuint n) const override { return const_cast<Atom&>(atoms[n]); }
    AtomID get_id(cuint n) override {
        if (n > atoms.size()) return AtomID();
        return AtomID(&atoms[n], n);
    }
    uint size() const override { return (uint)atoms.size(); }
    //! the records as the flat array the C ABI copies
    double* records() { return reinterpret_cast<double*>(atoms.data()); }
};

#endif
