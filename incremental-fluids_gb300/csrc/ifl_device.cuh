// ifl_device.cuh - device-side building blocks shared by the kernels.
//
// Everything here restates the reference's per-cell arithmetic with the same
// operation order (the library is compiled with --fmad=false, so the FP64 path
// is bit-identical to the reference built with -ffp-contract=off).
#pragma once
#include "ifl_internal.h"

namespace ifl {

// std::min / std::max forms (NaN handling follows the comparison).
template <typename T> __device__ __forceinline__ T smin(T a, T b) { return (b < a) ? b : a; }
template <typename T> __device__ __forceinline__ T smax(T a, T b) { return (a < b) ? b : a; }
__device__ __forceinline__ int sgn(double v) { return (0.0 < v) - (v < 0.0); }
__device__ __forceinline__ int nsgn(double v) { return v < 0.0 ? -1 : 1; }

__device__ __forceinline__ double length2(double x, double y) { return sqrt(x * x + y * y); }

// rotate(x, y, phi) of 4-solid-boundaries/Fluid.cpp:58-62 with c = cos(phi),
// s = sin(phi) supplied by the host.
__device__ __forceinline__ void rotate_cs(double &x, double &y, double c, double s) {
    double tx = x, ty = y;
    x = c * tx + s * ty;
    y = -s * tx + c * ty;
}

// SolidBox::distance / SolidSphere::distance (4-solid-boundaries/Fluid.cpp:158-169, 210-212)
__device__ __forceinline__ double body_distance(const DevBody &b, double x, double y) {
    if (b.type == 0) {
        x -= b.px;
        y -= b.py;
        rotate_cs(x, y, b.cneg, b.sneg);
        double dx = fabs(x) - b.sx * 0.5;
        double dy = fabs(y) - b.sy * 0.5;
        if (dx >= 0.0 || dy >= 0.0) return length2(smax(dx, 0.0), smax(dy, 0.0));
        return smax(dx, dy);
    }
    return length2(x - b.px, y - b.py) - b.sx * 0.5;
}

// closestSurfacePoint (4-solid-boundaries/Fluid.cpp:171-186, 214-227)
__device__ __forceinline__ void body_closest(const DevBody &b, double &x, double &y) {
    if (b.type == 0) {
        x -= b.px;
        y -= b.py;
        rotate_cs(x, y, b.cneg, b.sneg);
        double dx = fabs(x) - b.sx * 0.5;
        double dy = fabs(y) - b.sy * 0.5;
        if (dx > dy)
            x = nsgn(x) * 0.5 * b.sx;
        else
            y = nsgn(y) * 0.5 * b.sy;
        rotate_cs(x, y, b.cpos, b.spos);
        x += b.px;
        y += b.py;
    } else {
        x -= b.px;
        y -= b.py;
        rotate_cs(x, y, b.cneg, b.sneg);
        x /= b.sx;
        y /= b.sy;
        double r = length2(x, y);
        if (r < 1e-4) {
            x = 0.5;
            y = 0.0;
        } else {
            x /= 2.0 * r;
            y /= 2.0 * r;
        }
        x *= b.sx;
        y *= b.sy;
        rotate_cs(x, y, b.cpos, b.spos);
        x += b.px;
        y += b.py;
    }
}

// distanceNormal (4-solid-boundaries/Fluid.cpp:188-200, 229-240; the sphere
// rounds its radius through float)
__device__ __forceinline__ void body_normal(const DevBody &b, double &nx, double &ny, double x, double y) {
    if (b.type == 0) {
        x -= b.px;
        y -= b.py;
        rotate_cs(x, y, b.cneg, b.sneg);
        if (fabs(x) - b.sx * 0.5 > fabs(y) - b.sy * 0.5) {
            nx = nsgn(x);
            ny = 0.0;
        } else {
            nx = 0.0;
            ny = nsgn(y);
        }
        rotate_cs(nx, ny, b.cpos, b.spos);
    } else {
        x -= b.px;
        y -= b.py;
        float r = __double2float_rn(length2(x, y));
        if (r < 1e-4) {
            nx = 1.0;
            ny = 0.0;
        } else {
            nx = x / r;
            ny = y / r;
        }
    }
}

// SolidBody::velocityX/Y (4-solid-boundaries/Fluid.cpp:127-133)
__device__ __forceinline__ double body_vel_x(const DevBody &b, double /*x*/, double y) {
    return (b.py - y) * b.vth + b.vx;
}
__device__ __forceinline__ double body_vel_y(const DevBody &b, double x, double /*y*/) {
    return (x - b.px) * b.vth + b.vy;
}

// occupancy (7-variable-density/Fluid.cpp:60-102)
__device__ __forceinline__ double tri_occ(double out1, double in, double out2) {
    return 0.5 * in * in / ((out1 - in) * (out2 - in));
}
__device__ __forceinline__ double trap_occ(double out1, double out2, double in1, double in2) {
    return 0.5 * (-in1 / (out1 - in1) - in2 / (out2 - in2));
}
__device__ __forceinline__ double occupancy(double d11, double d12, double d21, double d22) {
    unsigned b = (d21 < 0.0 ? 8u : 0u) | (d22 < 0.0 ? 4u : 0u) | (d12 < 0.0 ? 2u : 0u) |
                 (d11 < 0.0 ? 1u : 0u);
    switch (b) {
    case 0x0: return 0.0;
    case 0x1: return tri_occ(d21, d11, d12);
    case 0x2: return tri_occ(d11, d12, d22);
    case 0x4: return tri_occ(d12, d22, d21);
    case 0x8: return tri_occ(d22, d21, d11);
    case 0xE: return 1.0 - tri_occ(-d21, -d11, -d12);
    case 0xD: return 1.0 - tri_occ(-d11, -d12, -d22);
    case 0xB: return 1.0 - tri_occ(-d12, -d22, -d21);
    case 0x7: return 1.0 - tri_occ(-d22, -d21, -d11);
    case 0x3: return trap_occ(d21, d22, d11, d12);
    case 0x6: return trap_occ(d11, d21, d12, d22);
    case 0x9: return trap_occ(d12, d22, d11, d21);
    case 0xC: return trap_occ(d11, d12, d21, d22);
    case 0x5: return tri_occ(d11, d12, d22) + tri_occ(d22, d21, d11);
    case 0xA: return tri_occ(d21, d11, d12) + tri_occ(d12, d22, d21);
    default: return 1.0;  // 0xF
    }
}

// cubicPulse (3-conjugate-gradients/Fluid.cpp:36-39)
__device__ __forceinline__ double cubic_pulse(double x) {
    x = smin(fabs(x), 1.0);
    return 1.0 - x * x * (3.0 - 2.0 * x);
}

template <typename F> __device__ __forceinline__ F lerp1(F a, F b, F x) { return a * (F(1.0) - x) + b * x; }

// FluidQuantity::lerp (3-conjugate-gradients/Fluid.cpp:121-133) on a pitched grid.
template <typename F>
__device__ __forceinline__ F q_lerp(const F *__restrict__ src, int P, int w, int h, F ox, F oy, F x, F y) {
    x = smin(smax(x - ox, F(0.0)), F(w) - F(1.001));
    y = smin(smax(y - oy, F(0.0)), F(h) - F(1.001));
    int ix = (int)x, iy = (int)y;
    x -= F(ix);
    y -= F(iy);
    const F *r0 = src + ix + (size_t)iy * P;
    F x00 = __ldg(r0), x10 = __ldg(r0 + 1);
    F x01 = __ldg(r0 + P), x11 = __ldg(r0 + P + 1);
    return lerp1(lerp1(x00, x10, x), lerp1(x01, x11, x), y);
}

// Bounded spin: the status word records a timeout and the caller proceeds
// (the result is then garbage, but nothing hangs and the host sees the flag).
constexpr long long kSpinLimit = 1ll << 26;

__device__ __forceinline__ unsigned ld_volatile(const unsigned *p) {
    return *(const volatile unsigned *)p;
}
__device__ __forceinline__ void st_volatile(unsigned *p, unsigned v) { *(volatile unsigned *)p = v; }

}  // namespace ifl
