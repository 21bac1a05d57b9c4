// Poisson noise for the pattern epilogue (the step of CTEMEBSD.f90:611-615).
//
// The reference draws from one sequential generator (noise.f90:136-217,
// idum = -1 at CTEMEBSD.f90:536) in pixel order, which no parallel
// implementation can reproduce draw for draw.  Here every pixel of every
// pattern has its own counter-based stream: Philox4x32-10 (Salmon, Moraes,
// Dror and Shaw, "Parallel random numbers: as easy as 1, 2, 3", SC 2011)
// keyed by the seed, with the counter (pattern index, pixel index), so the
// noise does not depend on launch shape, chunking or device.  The sampler
// is inversion by sequential search for means below kInversionMax and
// Hormann's transformed rejection with squeeze, PTRS ("The transformed
// rejection method for generating Poisson random variables", Insurance:
// Mathematics and Economics 12, 1993; valid for means >= 10) above.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace ebsd {

struct Philox4 {
    uint32_t v[4];
};

__device__ __forceinline__ Philox4 philox4x32_10(uint32_t c0, uint32_t c1, uint32_t c2,
                                                 uint32_t c3, uint32_t k0, uint32_t k1)
{
    const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;  // round multipliers
    const uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;  // key schedule (Weyl)
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        const uint32_t hi0 = __umulhi(M0, c0), lo0 = M0 * c0;
        const uint32_t hi1 = __umulhi(M1, c2), lo1 = M1 * c2;
        const uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
        c0 = n0;
        c1 = lo1;
        c2 = n2;
        c3 = lo0;
        k0 += W0;
        k1 += W1;
    }
    Philox4 out;
    out.v[0] = c0;
    out.v[1] = c1;
    out.v[2] = c2;
    out.v[3] = c3;
    return out;
}

// Uniform in (0, 1): 24 random bits, centred in their interval.
__device__ __forceinline__ float u01(uint32_t x)
{
    return ((float)(x >> 8) + 0.5f) * (1.0f / 16777216.0f);
}

// Per-pixel stream: four uniforms per Philox call; the call index is the
// fourth counter word, so a rejection loop draws fresh blocks.  The block
// is held in registers and read with selects (no local memory).
struct PixelRng {
    uint32_t c0, c1, c2, k0, k1, call;
    Philox4 blk;
    int used;
    __device__ PixelRng(uint64_t seed, uint64_t pattern, uint32_t pixel)
        : c0((uint32_t)pattern), c1((uint32_t)(pattern >> 32)), c2(pixel),
          k0((uint32_t)seed), k1((uint32_t)(seed >> 32)), call(0), used(4)
    {
    }
    // Draw the next block now (the block the next call of next() would
    // draw), so that code paths that diverge afterwards share its cost.
    __device__ void fill()
    {
        blk = philox4x32_10(c0, c1, c2, call++, k0, k1);
        used = 0;
    }
    __device__ float next()
    {
        if (used == 4) {
            blk = philox4x32_10(c0, c1, c2, call++, k0, k1);
            used = 0;
        }
        const uint32_t x = used == 0 ? blk.v[0] : used == 1 ? blk.v[1] : used == 2 ? blk.v[2]
                                                                                    : blk.v[3];
        ++used;
        return u01(x);
    }
};

// log k! for k = 0..15 (ln of the factorials).
__device__ __constant__ float c_log_fact[16] = {
    0.000000000e+00f, 0.000000000e+00f, 6.931471806e-01f, 1.791759469e+00f,
    3.178053830e+00f, 4.787491743e+00f, 6.579251212e+00f, 8.525161361e+00f,
    1.060460290e+01f, 1.280182748e+01f, 1.510441257e+01f, 1.750230785e+01f,
    1.998721450e+01f, 2.255216385e+01f, 2.519122118e+01f, 2.789927138e+01f};

// log of the Poisson probability p(k; lambda) = exp(-lambda) lambda^k / k!,
// without the cancellation of the direct form (whose terms grow like
// lambda log lambda).  For k >= 16, Stirling's series
//   log k! = k log k - k + log(2 pi k)/2 + 1/(12k) - 1/(360k^3) + ...
// gives log p = -lambda h(x) - log(2 pi k)/2 - 1/(12k) + 1/(360k^3),
// x = (k - lambda)/lambda, h(x) = (1+x) log(1+x) - x, summed as its power
// series sum_{n>=2} (-x)^n / (n (n-1)) (times -1 for odd n) near 0.
//
// The sampler only needs statistical accuracy: logarithms, exponentials and
// divides use the hardware intrinsics (__logf, __expf, __fdividef; errors of
// order 1e-6, far below what changes a distribution).  The pattern means sit
// around 10 at the reference's beam settings, so most warps run both the
// inversion and the PTRS branch and the cost of each shows.
__device__ __forceinline__ float log_poisson_pmf(float k, float lambda, float loglam)
{
    if (k < 16.0f) return -lambda + k * loglam - c_log_fact[(int)k];
    const float x = __fdividef(k - lambda, lambda);
    float h;
    if (fabsf(x) < 0.125f) {
        // x^2/2 - x^3/6 + x^4/12 - x^5/20 + x^6/30 - x^7/42 + x^8/56
        const float x2 = x * x;
        h = x2 * (0.5f + x * (-1.0f / 6.0f + x * (1.0f / 12.0f + x * (-1.0f / 20.0f +
             x * (1.0f / 30.0f + x * (-1.0f / 42.0f + x * (1.0f / 56.0f)))))));
    } else {
        h = (1.0f + x) * __logf(1.0f + x) - x;
    }
    const float ik = __fdividef(1.0f, k);
    return -lambda * h - 0.5f * __logf(6.28318531f * k) - ik * (1.0f / 12.0f) +
           ik * ik * ik * (1.0f / 360.0f);
}

// Inversion below this mean, PTRS from it on (PTRS needs means >= 10).  A
// warp runs every branch that one of its lanes takes, so where a pattern's
// means straddle the split both branches run; measured on 640x480 patterns
// over five intensity scales (means ~1 to ~100), a split at 10 is the best
// compromise: 20 or 30 gain 2-9 % at means near 10 and lose 13-25 % at
// means of 30-100, where the long sequential searches of the dim pixels
// hold up warps of PTRS draws.
constexpr float kInversionMax = 10.0f;

// One Poisson(lambda) draw.  lambda <= 0 (or NaN) gives 0.  rng is a fresh
// stream (nothing drawn yet): both samplers start with its first block,
// which is drawn here, before the lanes of a warp split between inversion
// and PTRS, so a warp whose pixels straddle kInversionMax (most of them at
// the reference's beam settings) runs the ten Philox rounds once, not once
// per branch; the uniforms are the same.
__device__ __forceinline__ float poisson_draw(float lambda, PixelRng& rng)
{
    rng.fill();
    if (!(lambda > 0.0f)) return 0.0f;
    if (lambda < kInversionMax) {
        // inversion: walk the cumulative distribution from k = 0.  Rounding
        // can leave the single-precision sum a little below 1; a u above it
        // ends the walk where the terms no longer move the sum (deep in the
        // tail, probability ~1e-7) instead of running on to the cap.
        const float u = rng.next();
        float p = __expf(-lambda), cdf = p;
        int k = 0;
        while (u > cdf && k < 200) {
            ++k;
            p *= __fdividef(lambda, (float)k);
            if (p <= 5.9604645e-8f * cdf) break;  // 2^-24 of the sum
            cdf += p;
        }
        return (float)k;
    }
    // PTRS, Hormann (1993), constants from the paper
    const float slam = sqrtf(lambda), loglam = __logf(lambda);
    const float b = 0.931f + 2.53f * slam;
    const float a = -0.059f + 0.02483f * b;
    const float loginvalpha = __logf(1.1239f + __fdividef(1.1328f, b - 3.4f));
    const float vr = 0.9277f - __fdividef(3.6224f, b - 2.0f);
    for (int it = 0; it < 64; ++it) {  // acceptance > 0.85 per try
        const float U = rng.next() - 0.5f;
        const float V = rng.next();
        const float us = 0.5f - fabsf(U);
        const float k = floorf((__fdividef(2.0f * a, us) + b) * U + lambda + 0.43f);
        if (us >= 0.07f && V <= vr) return k;
        if (k < 0.0f || (us < 0.013f && V > us)) continue;
        if (__logf(V) + loginvalpha - __logf(__fdividef(a, us * us) + b) <=
            log_poisson_pmf(k, lambda, loglam))
            return k;
    }
    return floorf(lambda + 0.5f);  // not reached in practice (p < 1e-50)
}

}  // namespace ebsd
