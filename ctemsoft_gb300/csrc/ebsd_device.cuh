// Device-side arithmetic of the EBSD pattern loop.
//
// Every translation unit that includes this file is compiled with
// -fmad=false and IEEE division/square root, so each float expression below
// is one correctly rounded binary32 operation per operator, evaluated left
// to right exactly as gfortran evaluates the cited Fortran.  Where a fused
// multiply-add is wanted it is written as fmaf() explicitly.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace ebsd {

// L2 eviction priorities for loads (PTX createpolicy / L2::cache_hint): the
// master pattern and the per-pixel detector tables are re-read by every
// orientation, so they are fetched with evict_last and outlive the
// streaming pattern stores (which are written evict-first).
__device__ __forceinline__ uint64_t l2_policy_evict_last()
{
    uint64_t pol;
    asm("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(pol));
    return pol;
}

__device__ __forceinline__ float4 ldg4_keep(const float4* p, uint64_t pol)
{
    float4 v;
    asm("ld.global.nc.L2::cache_hint.v4.f32 {%0, %1, %2, %3}, [%4], %5;"
                 : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
                 : "l"(p), "l"(pol));
    return v;
}

// Two binary32 values in one 64-bit register pair (low half first), for the
// packed FP32 instructions of sm_100 and later (PTX fma/mul/add .rn.f32x2):
// each half is one IEEE binary32 operation rounded to nearest, exactly the
// scalar operation's result, two per issued instruction.  The sums below
// that use them carry bins of even and odd index in the two halves.
typedef unsigned long long f2_t;

__device__ __forceinline__ f2_t f2_pack(float lo, float hi)
{
    f2_t r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
    return r;
}

__device__ __forceinline__ float f2_sum(f2_t v)  // lo + hi
{
    float lo, hi;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v));
    return lo + hi;
}

__device__ __forceinline__ f2_t f2_fma(f2_t a, f2_t b, f2_t c)
{
    f2_t d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}

__device__ __forceinline__ f2_t f2_mul(f2_t a, f2_t b)
{
    f2_t d;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}

// 128-bit read-only load with the L2 policy, as two pairs (x, y), (z, w).
__device__ __forceinline__ void ldg4_keep2(const float4* p, uint64_t pol, f2_t& lo, f2_t& hi)
{
    asm("ld.global.nc.L2::cache_hint.v2.b64 {%0, %1}, [%2], %3;"
        : "=l"(lo), "=l"(hi)
        : "l"(p), "l"(pol));
}

// qq3 = q (x) (0,r) (x) conjg(q), quaternions.f90:255-264,306-313 as used at
// CTEMEBSD.f90:577-586; returns the vector part.  The first product's terms
// with the zero scalar part of (0,r) are left out: 0*y is +-0 for finite y,
// and (+-0) - a = -a, (+-0) + a = a exactly for every a != 0, so only the
// sign of an exact-zero component can differ from the reference, which moves
// neither a Lambert cell nor a value.
__device__ __forceinline__ void rotate_direction(const float4 q, float rx, float ry, float rz,
                                                 float& d0, float& d1, float& d2)
{
    const float y0 = q.x, y1 = -q.y, y2 = -q.z, y3 = -q.w;   // conjg(q)
    const float t0 = -(rx * y1) - ry * y2 - rz * y3;           // quat_mult(qq, qq1)
    const float t1 = rx * y0 + ry * y3 - rz * y2;
    const float t2 = -(rx * y3) + ry * y0 + rz * y1;
    const float t3 = rx * y2 - ry * y1 + rz * y0;
    d0 = q.x * t1 + q.y * t0 + q.z * t3 - q.w * t2;           // quat_mult(qq2, t)
    d1 = q.x * t2 - q.y * t3 + q.z * t0 + q.w * t1;
    d2 = q.x * t3 + q.y * t2 - q.z * t1 + q.w * t0;
}

// dc = dc/sqrt(sum(dc**2)); if (dc(3) < 0) dc = -dc   (CTEMEBSD.f90:588-589)
__device__ __forceinline__ void normalize_fold(float& d0, float& d1, float& d2)
{
    float s = d0 * d0;
    s = s + d1 * d1;
    s = s + d2 * d2;
    s = sqrtf(s);
    d0 = d0 / s;
    d1 = d1 / s;
    d2 = d2 / s;
    if (d2 < 0.0f) {
        d0 = -d0;
        d1 = -d1;
        d2 = -d2;
    }
}

// Lambert2DSquareInverseSingle, Lambert.f90:405-436.  spi2 = sngl(LPs%sPi2).
// abs(x)/x * sqrt(.) is +-sqrt(.) exactly for x != 0, and x == 0 only
// reaches this branch together with y == 0, which |z| == 1 intercepts.
//
// accurate == false evaluates 1 - z as the reference does; near the poles
// that difference cancels (z within 1e-5 of 1 loses ~1% of 1 - z), which
// moves the Lambert point by up to ~1e-3 cells against a binary64
// evaluation.  accurate == true uses the identity 1 - z = (x^2+y^2)/(1+z)
// for unit vectors, which has no cancellation.
__device__ __forceinline__ void lambert_inverse(float x, float y, float z, float spi2,
                                                float& X, float& Y, bool accurate = false)
{
    float s = x * x;
    s = s + y * y;
    const float rxy = s;
    s = s + z * z;
    if (fabsf(1.0f - s) > 1.0e-6f || fabsf(z) == 1.0f) {
        X = 0.0f;
        Y = 0.0f;
        return;
    }
    const float omz = accurate ? rxy / (1.0f + z) : 1.0f - z;
    if (fabsf(y) <= fabsf(x)) {
        const float q = copysignf(sqrtf(2.0f * omz), x);
        X = q * spi2;
        Y = q * atanf(y / x) / spi2;
    } else {
        const float q = copysignf(sqrtf(2.0f * omz), y);
        X = q * atanf(x / y) / spi2;
        Y = q * spi2;
    }
}

// The square Lambert map of Lambert.f90:405-436 and its Jacobian with respect
// to (x, y, z), for the adjoint kernels.  The adjoint does not need the
// reference's rounding: the bilinear gather is continuous across cell edges,
// so a point placed an ulp differently changes the value only by rounding.
// So the map is evaluated in the cancellation-free form
// rho^2 = 2(1 - z) = 2(x^2 + y^2)/(1 + z) with the hardware reciprocal
// square root and fast divide (CUDA intrinsics, 2-ulp bounds) instead of the
// IEEE operations of lambert_inverse.  Zero where the map is intercepted
// (|z| = 1, non-unit input, or x = y = 0).
__device__ __forceinline__ void lambert_inverse_jac(float x, float y, float z, float spi2,
                                                    float& X, float& Y, float dX[3], float dY[3])
{
    float s = x * x;
    s = s + y * y;
    const float rxy = s;
    s = s + z * z;
    dX[0] = dX[1] = dX[2] = 0.0f;
    dY[0] = dY[1] = dY[2] = 0.0f;
    X = 0.0f;
    Y = 0.0f;
    if (fabsf(1.0f - s) > 1.0e-6f || fabsf(z) == 1.0f || !(rxy > 0.0f)) return;
    const bool xb = fabsf(y) <= fabsf(x);
    const float u = xb ? x : y, v = xb ? y : x;       // |v| <= |u|, u != 0
    const float t = __fdividef(2.0f * rxy, 1.0f + z);  // rho^2 (z >= 0 after the fold)
    const float irho = rsqrtf(t);
    const float rho = t * irho;
    const float sg = copysignf(1.0f, u);
    const float q = sg * rho;
    const float a = atanf(__fdividef(v, u));
    const float ispi2 = __fdividef(1.0f, spi2);
    const float along = q * spi2, across = q * a * ispi2;
    X = xb ? along : across;
    Y = xb ? across : along;
    const float f = sg * __fdividef(rho * ispi2, rxy);
    // d(along)/dz, d(across)/d(u, v, z)
    const float dal_z = -sg * spi2 * irho;
    const float dac_u = -f * v, dac_v = f * u, dac_z = -sg * a * irho * ispi2;
    if (xb) {  // along = X (u = x), across = Y (v = y)
        dX[2] = dal_z;
        dY[0] = dac_u;
        dY[1] = dac_v;
        dY[2] = dac_z;
    } else {   // along = Y (u = y), across = X (v = x)
        dY[2] = dal_z;
        dX[1] = dac_u;
        dX[0] = dac_v;
        dX[2] = dac_z;
    }
}

// Cell index and bilinear fractions, CTEMEBSD.f90:593-598:
// nix = int(npx + ixy) - npx (float add, then truncation), dx = ixy - nix.
// Returns the 0-based grid column of the lower corner, clamped to the grid.
//
// The truncation is taken without the float/integer conversion instructions
// (which run on a slower pipe): t = npx + ixy is the reference's binary32
// sum; for 0 <= t < 2^23, adding 2^23 rounded toward zero leaves 2^23 +
// int(t) exactly, whose low mantissa bits are int(t), and subtracting 2^23
// again gives int(t) as an exact float, so dx = ixy - (int(t) - npx) is the
// reference's value bit for bit.  t lies in that range: |ixy| <= npx up to a
// few ulps (|X|, |Y| <= sqrt(pi/2) for unit directions, and the intercepted
// ones map to 0), so t > -1, where int() gives 0 as max(t, 0) does.
// (+0.8 % at 640x480 against cvt.rzi / cvt.rn.)
__device__ __forceinline__ int lambert_cell(float ixy, int np, float& d, int& ni)
{
    const float t = (float)np + ixy;
    const float tt = __fadd_rz(fmaxf(t, 0.0f), 8388608.0f);  // 2^23 + int(t)
    const int it = __float_as_int(tt) - 0x4B000000;          // int(t)
    ni = it - np;
    d = ixy - ((tt - 8388608.0f) - (float)np);
    return min(it, 2 * np);
}

}  // namespace ebsd
