// Minimal single-rank stand-in for the FDPS `PS` namespace.
//
// TEST INFRASTRUCTURE ONLY.  FDPS (a git submodule of GPLUM) is absent from
// the reference tree, so GPLUM's own hot-path headers (gravity_kernel.hpp,
// cutfunc.h, particle.h, gravity_soft.h, neighbor.h, hard.h, hermite.h,
// gravity_hard.h, kepler.h, collisionA/B.h, energy.h) are compiled unchanged
// against this file to produce the reference build under oracle/_ref/.
//
// Only what those headers name is provided: the scalar typedefs, Vector3 with
// FDPS semantics (operator* between vectors is the dot product, assignment
// from a scalar broadcasts), the symmetric 3x3 matrix, quadrupole moments /
// superparticles (quad = sum m (x-c)(x-c)^T, not traceless, as the EP-SP
// functor expects), and identity single-rank Comm wrappers.
#pragma once

#include <cassert>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <iostream>
#include <fstream>
#include <sstream>
#include <iomanip>
#include <limits>
#include <string>
#include <vector>
#include <map>
#include <algorithm>
#include <sys/time.h>

namespace ParticleSimulator {

typedef int32_t  S32;
typedef int64_t  S64;
typedef uint32_t U32;
typedef uint64_t U64;
typedef float    F32;
typedef double   F64;

template <class T>
class Vector3 {
public:
    T x, y, z;
    Vector3() : x(T(0)), y(T(0)), z(T(0)) {}
    Vector3(const T a, const T b, const T c) : x(a), y(b), z(c) {}
    Vector3(const T s) : x(s), y(s), z(s) {}
    template <class U>
    Vector3(const Vector3<U> &v) : x(T(v.x)), y(T(v.y)), z(T(v.z)) {}
    Vector3 &operator=(const T s) { x = y = z = s; return *this; }
    template <class U>
    Vector3 &operator=(const Vector3<U> &v) { x = T(v.x); y = T(v.y); z = T(v.z); return *this; }

    Vector3 operator+(const Vector3 &v) const { return Vector3(x + v.x, y + v.y, z + v.z); }
    Vector3 operator-(const Vector3 &v) const { return Vector3(x - v.x, y - v.y, z - v.z); }
    Vector3 operator-() const { return Vector3(-x, -y, -z); }
    const Vector3 &operator+() const { return *this; }
    Vector3 operator*(const T s) const { return Vector3(x * s, y * s, z * s); }
    friend Vector3 operator*(const T s, const Vector3 &v) { return Vector3(s * v.x, s * v.y, s * v.z); }
    Vector3 operator/(const T s) const { return Vector3(x / s, y / s, z / s); }
    // dot product, evaluated left to right
    T operator*(const Vector3 &v) const { return x * v.x + y * v.y + z * v.z; }
    Vector3 operator^(const Vector3 &v) const {
        return Vector3(y * v.z - z * v.y, z * v.x - x * v.z, x * v.y - y * v.x);
    }
    Vector3 &operator+=(const Vector3 &v) { x += v.x; y += v.y; z += v.z; return *this; }
    Vector3 &operator-=(const Vector3 &v) { x -= v.x; y -= v.y; z -= v.z; return *this; }
    Vector3 &operator*=(const T s) { x *= s; y *= s; z *= s; return *this; }
    Vector3 &operator/=(const T s) { x /= s; y /= s; z /= s; return *this; }
    bool operator==(const Vector3 &v) const { return x == v.x && y == v.y && z == v.z; }
    bool operator!=(const Vector3 &v) const { return !(*this == v); }
    T &operator[](const int i) { return i == 0 ? x : (i == 1 ? y : z); }
    const T &operator[](const int i) const { return i == 0 ? x : (i == 1 ? y : z); }
    friend std::ostream &operator<<(std::ostream &c, const Vector3 &u) {
        c << u.x << "   " << u.y << "    " << u.z;
        return c;
    }
};

template <class T>
class MatrixSym3 {
public:
    T xx, yy, zz, xy, xz, yz;
    MatrixSym3() : xx(0), yy(0), zz(0), xy(0), xz(0), yz(0) {}
    MatrixSym3(const T s) : xx(s), yy(s), zz(s), xy(s), xz(s), yz(s) {}
    MatrixSym3 &operator=(const T s) { xx = yy = zz = xy = xz = yz = s; return *this; }
    T getTrace() const { return xx + yy + zz; }
    friend std::ostream &operator<<(std::ostream &c, const MatrixSym3 &m) {
        c << m.xx << " " << m.yy << " " << m.zz << " " << m.xy << " " << m.xz << " " << m.yz;
        return c;
    }
};

typedef Vector3<F32> F32vec;
typedef Vector3<F64> F64vec;
typedef MatrixSym3<F64> F64mat;

// Monopole / quadrupole moments and superparticles.  quad is the raw second
// moment about the centre of mass: sum m (x-c)(x-c)^T.
class MomentMonopole {
public:
    F64 mass;
    F64vec pos;
    MomentMonopole() : mass(0), pos(0.) {}
    MomentMonopole(const F64 m, const F64vec &p) : mass(m), pos(p) {}
    void init() { mass = 0.; pos = 0.; }
    F64vec getPos() const { return pos; }
    F64 getCharge() const { return mass; }
    template <class Tepj> void accumulateAtLeaf(const Tepj &epj) {
        mass += epj.getCharge();
        pos += epj.getCharge() * epj.getPos();
    }
    template <class Tepj> void accumulateAtLeaf2(const Tepj &) {}
    void accumulate(const MomentMonopole &m) { mass += m.mass; pos += m.mass * m.pos; }
    void accumulate2(const MomentMonopole &) {}
    void set() { pos = (mass != 0.) ? pos / mass : F64vec(0.); }
};

class MomentQuadrupole {
public:
    F64 mass;
    F64vec pos;
    F64mat quad;
    MomentQuadrupole() : mass(0), pos(0.), quad(0.) {}
    MomentQuadrupole(const F64 m, const F64vec &p, const F64mat &q) : mass(m), pos(p), quad(q) {}
    void init() { mass = 0.; pos = 0.; quad = 0.; }
    F64vec getPos() const { return pos; }
    F64 getCharge() const { return mass; }
    template <class Tepj> void accumulateAtLeaf(const Tepj &epj) {
        mass += epj.getCharge();
        pos += epj.getCharge() * epj.getPos();
    }
    template <class Tepj> void accumulateAtLeaf2(const Tepj &epj) {
        F64 c = epj.getCharge();
        F64vec d = epj.getPos() - pos;
        F64 cx = c * d.x, cy = c * d.y, cz = c * d.z;
        quad.xx += cx * d.x; quad.yy += cy * d.y; quad.zz += cz * d.z;
        quad.xy += cx * d.y; quad.xz += cx * d.z; quad.yz += cy * d.z;
    }
    void accumulate(const MomentQuadrupole &m) { mass += m.mass; pos += m.mass * m.pos; }
    void accumulate2(const MomentQuadrupole &m) {
        F64 c = m.mass;
        F64vec d = m.pos - pos;
        F64 cx = c * d.x, cy = c * d.y, cz = c * d.z;
        quad.xx += cx * d.x + m.quad.xx; quad.yy += cy * d.y + m.quad.yy;
        quad.zz += cz * d.z + m.quad.zz; quad.xy += cx * d.y + m.quad.xy;
        quad.xz += cx * d.z + m.quad.xz; quad.yz += cy * d.z + m.quad.yz;
    }
    void set() { pos = (mass != 0.) ? pos / mass : F64vec(0.); }
};

class SPJMonopole {
public:
    F64 mass;
    F64vec pos;
    F64 getCharge() const { return mass; }
    F64vec getPos() const { return pos; }
    void copyFromMoment(const MomentMonopole &m) { mass = m.mass; pos = m.pos; }
    void clear() { mass = 0.; pos = 0.; }
    MomentMonopole convertToMoment() const { return MomentMonopole(mass, pos); }
};

class SPJQuadrupole {
public:
    F64 mass;
    F64vec pos;
    F64mat quad;
    F64 getCharge() const { return mass; }
    F64vec getPos() const { return pos; }
    void copyFromMoment(const MomentQuadrupole &m) { mass = m.mass; pos = m.pos; quad = m.quad; }
    void clear() { mass = 0.; pos = 0.; quad = 0.; }
    MomentQuadrupole convertToMoment() const { return MomentQuadrupole(mass, pos, quad); }
};

inline F64 GetWtime() {
    struct timeval tv;
    gettimeofday(&tv, nullptr);
    return double(tv.tv_sec) + double(tv.tv_usec) * 1e-6;
}

inline void Abort(const S32 err = -1) {
    std::fprintf(stderr, "PS::Abort(%d) called\n", err);
    std::abort();
}

// Domain decomposition is a single box on one rank; only named by time.h.
class DomainInfo {
public:
    F64 getUsedTime() const { return 0.; }
};

inline void Initialize(int &, char **&) {}
inline void Finalize() {}

// single rank: every collective is the identity
namespace Comm {
inline S32 getRank() { return 0; }
inline S32 getNumberOfProc() { return 1; }
inline S32 getNumberOfThread() { return 1; }
inline S32 getThreadNum() { return 0; }
inline void barrier() {}
template <class T> inline T getSum(const T &v) { return v; }
template <class T> inline T getMaxValue(const T &v) { return v; }
template <class T> inline T getMinValue(const T &v) { return v; }
template <class T> inline void broadcast(T *, const S32, const S32 = 0) {}
template <class T> inline void gather(const T *src, const S32 n, T *dst) {
    for (S32 i = 0; i < n; i++) dst[i] = src[i];
}
template <class T> inline void gatherV(const T *src, const S32 n, T *dst, const S32 *, const S32 *) {
    for (S32 i = 0; i < n; i++) dst[i] = src[i];
}
template <class T> inline void scatterV(const T *src, const S32 *n, const S32 *, T *dst, const S32 = 0) {
    for (S32 i = 0; i < n[0]; i++) dst[i] = src[i];
}
inline bool synchronizeConditionalBranchOR(const bool v) { return v; }
}  // namespace Comm

}  // namespace ParticleSimulator

namespace PS = ParticleSimulator;
