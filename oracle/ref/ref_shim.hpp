// Minimal stand-ins for the FDPS and PeTar types that the reference's force
// functors (src/soft_force.hpp) and SIMD kernels
// (src/phantomquad_for_p3t_x86.hpp) touch, so those reference headers compile
// on their own.  FDPS (the provider of PS::*) is not part of the reference
// tree.  Only the members the functors read or write exist here; field
// meanings follow src/soft_ptcl.hpp:4-24 (ForceSoft), :271-308 (EPISoft),
// :311-376 (EPJSoft) and FDPS's SPJQuadrupole (mass, pos, quad).
#pragma once
#include <algorithm>
#include <cassert>
#include <cmath>
#include <cstdint>
#include <iostream>

namespace PS {
typedef int S32;
typedef long long S64;
typedef double F64;
typedef float F32;

struct F64vec {
    double x, y, z;
    F64vec() : x(0), y(0), z(0) {}
    F64vec(double v) : x(v), y(v), z(v) {}
    F64vec(double a, double b, double c) : x(a), y(b), z(c) {}
    F64vec operator+(const F64vec& u) const { return F64vec(x + u.x, y + u.y, z + u.z); }
    F64vec operator-(const F64vec& u) const { return F64vec(x - u.x, y - u.y, z - u.z); }
    // Dot product, evaluated left to right as ((x*x) + (y*y)) + (z*z).
    double operator*(const F64vec& u) const { return x * u.x + y * u.y + z * u.z; }
    F64vec& operator+=(const F64vec& u) { x += u.x; y += u.y; z += u.z; return *this; }
    F64vec& operator-=(const F64vec& u) { x -= u.x; y -= u.y; z -= u.z; return *this; }
    double& operator[](int k) { return (&x)[k]; }
    const double& operator[](int k) const { return (&x)[k]; }
};
inline F64vec operator*(double s, const F64vec& v) { return F64vec(s * v.x, s * v.y, s * v.z); }

struct F64mat {
    double xx, yy, zz, xy, xz, yz;
    double getTrace() const { return xx + yy + zz; }
};
}  // namespace PS

class ForceSoft {
public:
    PS::F64vec acc;
    PS::F64 pot;
#ifdef KDKDK_4TH
    PS::F64vec acorr;
#endif
    PS::S64 n_ngb;
    static PS::F64 grav_const;
#ifdef KDKDK_4TH
    void clear() { acc = 0.0; pot = 0.0; acorr = 0.0; n_ngb = 0; }
#else
    void clear() { acc = 0.0; pot = 0.0; n_ngb = 0; }
#endif
};

class EPISoft {
public:
    PS::S64 id;
    PS::F64vec pos;
    PS::F64 r_search;
    PS::S32 rank_org;
    PS::S32 type;
#ifdef KDKDK_4TH
    PS::F64vec acc;
#endif
    static PS::F64 eps;
    static PS::F64 r_out;
    PS::F64vec getPos() const { return pos; }
};

class EPJSoft {
public:
    PS::S64 id;
    PS::F64 mass;
    PS::F64vec pos;
#ifdef KDKDK_4TH
    PS::F64vec acc;
#endif
    PS::F64 r_search;
    PS::F64vec getPos() const { return pos; }
    PS::F64 getCharge() const { return mass; }
};

class SPJSoft {
public:
    PS::F64 mass;
    PS::F64vec pos;
    PS::F64mat quad;
    PS::F64vec getPos() const { return pos; }
    PS::F64 getCharge() const { return mass; }
};
