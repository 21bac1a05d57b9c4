// The EBSD pattern loop on sm_103a: CTEMEBSD.f90:573-658.
//
// One CTA covers a 32 x tile_y block of detector pixels (one warp per
// detector row segment, so pattern stores are 128-byte coalesced) for a run
// of orientations.  Each thread loads its pixel's direction cosine and its
// NV float4 vectors of energy weights once and reuses them for every
// orientation of the run.  Per orientation it rotates the direction,
// projects it with the square Lambert map, and gathers the four master
// nodes around it: the master is stored energy-fastest (NV float4 per
// node), so one corner's bins arrive in NV 128-bit read-only loads that hit
// the L2-resident (persisting) master.
//
// Arithmetic follows the reference operation by operation (the TU is
// compiled with -fmad=false, IEEE div/sqrt): the geometry of :577-598, the
// column-major block sums of :636 and powf for 'gam'.  The reference-order
// variant (STRICT) also keeps the summation order of :600-604 and the
// binary64 prefactor multiply of :608; the default takes the gather as fused
// dot products, the prefactor multiply in binary32 and the hardware __powf,
// each within a few ulps.  Only atanf and the power function are CUDA's own.
#include "ebsd_device.cuh"
#include "ebsd_internal.h"
#include "ebsd_noise.cuh"

namespace ebsd {

namespace {

__device__ __forceinline__ float4 ldg4(const float4* p) { return __ldg(p); }

// 'gam' scaling, pattern**gammavalue (CTEMEBSD.f90:647-649).  The
// reference-order variant (STRICT) calls powf; the default takes the
// hardware exp2/log2 form (__powf, a few ulps) for positive values, 6 % of
// the kernel's time at 640x480 against parity gates of 1e-5 (FP64) and
// 1e-4 (reference).  fast: the exponent is positive, finite and not an
// integer (the launch's own flag, e.g. the reference's 0.33), for which
// __powf has powf's special values for every x (+-0 -> +0, x < 0 -> NaN,
// +inf -> +inf, NaN -> NaN), so no per-pixel test is needed: the test and
// its powf fallback cost 2.8 % at 640x480.
template <bool STRICT>
__device__ __forceinline__ float gamma_pow(float x, float g, bool fast)
{
    if (!STRICT && fast) return __powf(x, g);
    if (!STRICT && x > 0.0f) return __powf(x, g);
    return powf(x, g);
}

// Sum over the window of W(k) * bilinear(sr(.,.,k)), the loop body of
// CTEMEBSD.f90:600-604.  STRICT evaluates it in the reference's own order
// (((s00*dxm)*dym + (s10*dx)*dym + ...) per bin, accumulated bin by bin,
// no fused operations).  Otherwise the same sum is taken as four dot
// products of the weights with the four corner vectors, each accumulated
// with fused multiply-adds, then combined with the bilinear corner weights:
// about a third of the arithmetic, and no less accurate.
template <int NV, bool STRICT>
__device__ __forceinline__ float gather_pixel(const float4* __restrict__ master, int gx,
                                              int ix0, int iy0, int ix1, int iy1, float dx,
                                              float dy, const float4 (&w)[NV], uint64_t pol)
{
    const float dxm = 1.0f - dx, dym = 1.0f - dy;
    // node offsets in 32 bits: ebsd_set_master keeps the interleaved master
    // below 2^31 float4
    const float4* m00 = master + (uint32_t)(iy0 * gx + ix0) * (uint32_t)NV;
    const float4* m10 = master + (uint32_t)(iy0 * gx + ix1) * (uint32_t)NV;
    const float4* m01 = master + (uint32_t)(iy1 * gx + ix0) * (uint32_t)NV;
    const float4* m11 = master + (uint32_t)(iy1 * gx + ix1) * (uint32_t)NV;
    if (STRICT) {
        float acc = 0.0f;
#pragma unroll
        for (int c = 0; c < NV; ++c) {
            const float4 a = ldg4_keep(m00 + c, pol), b = ldg4_keep(m10 + c, pol),
                         e = ldg4_keep(m01 + c, pol), f = ldg4_keep(m11 + c, pol);
            acc = acc + w[c].x * (a.x * dxm * dym + b.x * dx * dym + e.x * dxm * dy + f.x * dx * dy);
            acc = acc + w[c].y * (a.y * dxm * dym + b.y * dx * dym + e.y * dxm * dy + f.y * dx * dy);
            acc = acc + w[c].z * (a.z * dxm * dym + b.z * dx * dym + e.z * dxm * dy + f.z * dx * dy);
            acc = acc + w[c].w * (a.w * dxm * dym + b.w * dx * dym + e.w * dxm * dy + f.w * dx * dy);
        }
        return acc;
    }
    // the four dot products on packed pairs of bins (even bins in the low
    // halves, odd in the high), two fused multiply-adds per instruction
    f2_t c00 = 0, c10 = 0, c01 = 0, c11 = 0;  // +0.0f pairs
#pragma unroll
    for (int c = 0; c < NV; ++c) {
        f2_t a0, a1, b0, b1, e0, e1, f0, f1;
        ldg4_keep2(m00 + c, pol, a0, a1);
        ldg4_keep2(m10 + c, pol, b0, b1);
        ldg4_keep2(m01 + c, pol, e0, e1);
        ldg4_keep2(m11 + c, pol, f0, f1);
        const f2_t w0 = f2_pack(w[c].x, w[c].y), w1 = f2_pack(w[c].z, w[c].w);
        c00 = f2_fma(w1, a1, f2_fma(w0, a0, c00));
        c10 = f2_fma(w1, b1, f2_fma(w0, b0, c10));
        c01 = f2_fma(w1, e1, f2_fma(w0, e0, c01));
        c11 = f2_fma(w1, f1, f2_fma(w0, f0, c11));
    }
    return fmaf(f2_sum(c00), dxm * dym,
                fmaf(f2_sum(c10), dx * dym, fmaf(f2_sum(c01), dxm * dy, f2_sum(c11) * (dx * dy))));
}

// Sum of the B x B binning block (B = 2 or 4) held by a warp of 32/B x B
// lanes (lane = row * 32/B + column).  STRICT: each block's top-left lane
// adds the B^2 values in the order of CTEMEBSD.f90:636 (x fastest).
// Otherwise a butterfly over the block's columns, then its rows, leaves the
// block total in every lane of the block.
template <int B, bool STRICT>
__device__ __forceinline__ float block_sum(float v, int lane)
{
    constexpr int BW = 32 / B;
    if (STRICT) {
        float s = 0.0f;
#pragma unroll
        for (int jj = 0; jj < B; ++jj)
#pragma unroll
            for (int ii = 0; ii < B; ++ii)
                s = s + __shfl_sync(0xffffffffu, v, (lane + jj * BW + ii) & 31);
        return s;
    }
#pragma unroll
    for (int o = 1; o < B; o <<= 1) v = v + __shfl_xor_sync(0xffffffffu, v, o);
#pragma unroll
    for (int o = 1; o < B; o <<= 1) v = v + __shfl_xor_sync(0xffffffffu, v, o * BW);
    return v;
}

// Rotated, projected and scaled Lambert coordinates of one pixel for one
// orientation (CTEMEBSD.f90:584-591).
__device__ __forceinline__ void pixel_lambert(const float4 q, const float4 r, float scl,
                                              float spi2, bool accurate, float& ixy0,
                                              float& ixy1)
{
    float d0, d1, d2;
    rotate_direction(q, r.x, r.y, r.z, d0, d1, d2);
    normalize_fold(d0, d1, d2);
    float X, Y;
    lambert_inverse(d0, d1, d2, spi2, X, Y, accurate);
    ixy0 = scl * X;
    ixy1 = scl * Y;
}

// Binary64 geometry of one pixel for one orientation: the FP64
// re-evaluation of CTEMEBSD.f90:584-598 (the rotation, normalisation and fold
// of :584-589, Lambert2DSquareInverseDouble of Lambert.f90:452-483, the cell
// of :593-598) from the binary64 detector direction (rx, ry, rz); the
// bilinear fractions are rounded once to binary32.  A single-precision
// Lambert coordinate near |ixy| = npx = 500 resolves 3e-5 of a cell, which
// on a sharp master moves a pixel by ~1e-4 of the pattern maximum; here the
// coordinate carries binary64 accuracy.
__device__ __forceinline__ void pixel_cell64(const float4 q, double rx, double ry, double rz,
                                             double scl, int npx, int npy, int& ix0, int& iy0,
                                             float& fdx, float& fdy)
{
    const double q0 = q.x, q1 = q.y, q2 = q.z, q3 = q.w;
    const double y1 = -q1, y2 = -q2, y3 = -q3;                 // conjg(q)
    const double t0 = -(rx * y1) - ry * y2 - rz * y3;          // (0, r) (x) conjg(q)
    const double t1 = rx * q0 + ry * y3 - rz * y2;
    const double t2 = -(rx * y3) + ry * q0 + rz * y1;
    const double t3 = rx * y2 - ry * y1 + rz * q0;
    double d0 = q0 * t1 + q1 * t0 + q2 * t3 - q3 * t2;         // q (x) t, vector part
    double d1 = q0 * t2 - q1 * t3 + q2 * t0 + q3 * t1;
    double d2 = q0 * t3 + q1 * t2 - q2 * t1 + q3 * t0;
    // binary64 divides and the arctangent run on GB300's slow binary64
    // pipe: one reciprocal normalises (within an ulp of three divides), and
    // 1/spi2 is a constant
    const double in = 1.0 / sqrt(d0 * d0 + d1 * d1 + d2 * d2);
    d0 = d0 * in;
    d1 = d1 * in;
    d2 = d2 * in;
    if (d2 < 0.0) {
        d0 = -d0;
        d1 = -d1;
        d2 = -d2;
    }
    const double spi2 = 0.88622692545275801365;   // sqrt(pi)/2
    const double ispi2 = 1.12837916709551257390;  // 2/sqrt(pi)
    double X = 0.0, Y = 0.0;
    const double s2 = d0 * d0 + d1 * d1 + d2 * d2;
    if (!(fabs(1.0 - s2) > 1.0e-12) && fabs(d2) != 1.0) {
        if (fabs(d1) <= fabs(d0)) {
            const double qq = copysign(sqrt(2.0 * (1.0 - d2)), d0);
            X = qq * spi2;
            Y = qq * atan(d1 / d0) * ispi2;
        } else {
            const double qq = copysign(sqrt(2.0 * (1.0 - d2)), d1);
            X = qq * atan(d0 / d1) * ispi2;
            Y = qq * spi2;
        }
    }
    const double ixy0 = scl * X, ixy1 = scl * Y;
    const int nix = (int)((double)npx + ixy0) - npx;
    const int niy = (int)((double)npy + ixy1) - npy;
    fdx = (float)(ixy0 - (double)nix);
    fdy = (float)(ixy1 - (double)niy);
    ix0 = min(max(nix + npx, 0), 2 * npx);
    iy0 = min(max(niy + npy, 0), 2 * npy);
}

// One work item: the 32 x tile_y pixels of tile t for orientations
// [o_begin, o_begin + opc).  `tile` is shared scratch of tile_y x 33 floats.
// BIN8: the variant for 8x8-binned records outside the reference-order mode
// (its pair barriers are kept out of the other variants, where their
// reservation would cost occupancy).  CELLS: the same kernel also stores
// each pixel's Lambert cell and coordinates (prm.nix, niy, ixy0, ixy1, one
// value per orientation and detector pixel) -- a diagnostic instantiation
// of this template, so that cell parity is read out of the code that makes
// the patterns.  G64: the pixel geometry in binary64 (pixel_cell64, option
// lambert_accurate = 2).
template <int NV, bool STRICT, bool NOISE, bool BIN8 = false, bool CELLS = false,
          bool G64 = false>
__device__ __forceinline__ void forward_tile(const FwdParams& prm, int tile_y, int tiles_x, int t,
                                             int64_t o_begin, int opc, float* tile, int bw)
{
    const int tid = threadIdx.x;
    const bool binned = prm.mode != EBSD_SCALING_NOT && prm.binning > 1;
    const int b = prm.binning;
    // Each warp covers a bw x (32 / bw) block of the tile (bw = 16 or 32).
    // A 16 x 2 block of detector pixels gathers from a more compact patch of
    // the master than a 32 x 1 row, so a warp's loads touch fewer cache
    // lines (1-3 % faster at 640x480) while its stores stay whole 64-byte
    // runs; stores into mapped host memory take whole 128-byte rows.  When
    // the record is binned 2x2 or 4x4 the warp block is one row of binning
    // blocks (16 x 2, 8 x 4), which are then summed within the warp.
    if (binned && b <= 4) bw = 32 / b;
    if (BIN8) bw = 8;  // an 8x8 block is two 8 x 4 warps
    const int bh = 32 / bw, wpr = kTileX / bw;
    const int lane = tid & 31, wid = tid >> 5;
    int lx = lane % bw, ly = lane / bw;
    if (!binned && bw == 16) {
        // each quarter-warp (the lanes whose 128-bit loads the L1 serves
        // together) a 4 x 2 block: its gathers span fewer cache lines than
        // an 8 x 1 row (4 % faster at 640x480)
        lx = (lane >> 3) * 4 + (lane & 3);
        ly = (lane >> 2) & 1;
    }
    const int tx = (wid % wpr) * bw + lx, ty = (wid / wpr) * bh + ly;
    const int x = (t % tiles_x) * kTileX + tx;
    const int y = (t / tiles_x) * tile_y + ty;
    const bool inside = x < prm.numsx && y < prm.numsy;
    const int p = y * prm.numsx + x;

    const uint64_t pol = l2_policy_evict_last();
    float4 r = make_float4(0.0f, 0.0f, 1.0f, 0.0f);
    float4 w[NV];
#pragma unroll
    for (int c = 0; c < NV; ++c) w[c] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    double r64x = 0.0, r64y = 0.0, r64z = 1.0;
    if (G64 && inside) {
        r64x = prm.rg64[p];
        r64y = prm.rg64[prm.P + p];
        r64z = prm.rg64[2 * (int64_t)prm.P + p];
    }
    if (inside) {
        r = ldg4_keep(prm.rg + p, pol);
#pragma unroll
        for (int c = 0; c < NV; ++c) w[c] = ldg4_keep(prm.W + (int64_t)c * prm.P + p, pol);
    }
    const int64_t rec = (int64_t)prm.out_nx * prm.out_ny;
    const float pref32 = (float)prm.prefactor;

    int64_t o_end = o_begin + opc;
    if (o_end > prm.n) o_end = prm.n;
    // two orientations per loop trip: the geometry of one overlaps the other's
    // gather (640x480: +0.5 %; four per trip take 56 registers, -15 %).  Not
    // for the noise variant (100 registers instead of 64 at two: -29 %) nor
    // the binary64-geometry and cells variants.
    constexpr int kUnroll = (NOISE || G64 || CELLS) ? 1 : 2;
#pragma unroll kUnroll
    for (int64_t o = o_begin; o < o_end; ++o) {
        float val = 0.0f;
        if (inside) {
            const float4 q = ldg4(prm.quats + o);
            float dx, dy;
            int ix0, iy0;
            float ixy0 = 0.0f, ixy1 = 0.0f;
            int nix = 0, niy = 0;
            if (G64) {
                pixel_cell64(q, r64x, r64y, r64z, prm.scl64, prm.npx, prm.npy, ix0, iy0, dx, dy);
            } else {
                pixel_lambert(q, r, prm.scl, prm.spi2, prm.accurate != 0, ixy0, ixy1);
                ix0 = lambert_cell(ixy0, prm.npx, dx, nix);
                iy0 = lambert_cell(ixy1, prm.npy, dy, niy);
            }
            const int ix1 = min(ix0 + 1, 2 * prm.npx), iy1 = min(iy0 + 1, 2 * prm.npy);
            if (CELLS) {
                const int64_t ci = o * (int64_t)prm.P + p;
                prm.nix[ci] = nix;
                prm.niy[ci] = niy;
                prm.ixy0[ci] = ixy0;
                prm.ixy1[ci] = ixy1;
            }
            const float acc =
                gather_pixel<NV, STRICT>(prm.master, prm.gx, ix0, iy0, ix1, iy1, dx, dy, w, pol);
            // :608 -- binary64 in the reference order; otherwise one binary32
            // multiply by the prefactor rounded once (within an ulp of the
            // binary64 product; 4 % faster at 640x480 than the slow FP64 pipe)
            val = STRICT ? (float)(prm.prefactor * (double)acc) : acc * pref32;
            if (NOISE) {                                                     // :611-615
                PixelRng rng(prm.seed, (uint64_t)(prm.o_offset + o), (uint32_t)p);
                val = poisson_draw(val, rng);
            }
        }
        if (!binned) {
            if (prm.mode == EBSD_SCALING_GAM)
                val = gamma_pow<STRICT>(val, prm.gammavalue, prm.gamma_fast);
            if (inside) __stcs(prm.out + o * rec + p, val);
        } else if (b <= 4) {
            // whole blocks within the warp: no CTA barrier
            float s = b == 2 ? block_sum<2, STRICT>(val, lane) : block_sum<4, STRICT>(val, lane);
            if (lane < bw && (lane & (b - 1)) == 0) {                        // top-left lanes
                s = s * prm.bindx;                                           // :640
                if (prm.mode == EBSD_SCALING_GAM)
                    s = gamma_pow<STRICT>(s, prm.gammavalue, prm.gamma_fast);
                const int X = ((t % tiles_x) * kTileX + tx) / b;
                const int Y = ((t / tiles_x) * tile_y + ty) / b;
                if (X < prm.out_nx && Y < prm.out_ny)
                    __stcs(prm.out + o * rec + (int64_t)Y * prm.out_nx + X, s);
            }
        } else if (BIN8) {
            // 8x8 blocks: each 8 x 4 warp sums its half by a butterfly; the
            // lower warp hands its half to the upper one through shared
            // memory (slots alternate with the orientation) and the pair
            // meets at its own named barrier, not the CTA's
            float sh = val;
#pragma unroll
            for (int m = 1; m < 32; m <<= 1) sh = sh + __shfl_xor_sync(0xffffffffu, sh, m);
            const int rgrp = wid / wpr;                          // 4-row group of the tile
            const int pair = (rgrp >> 1) * wpr + wid % wpr;      // 8x8 block within the tile
            float* slot = tile + ((int)(o & 1) * 32 + pair);
            if ((rgrp & 1) && lane == 0) *slot = sh;
            asm volatile("bar.sync %0, 64;" ::"r"(1 + pair) : "memory");
            if (!(rgrp & 1) && lane == 0) {
                float sb = sh + *slot;
                sb = sb * prm.bindx;                                         // :640
                if (prm.mode == EBSD_SCALING_GAM)
                    sb = gamma_pow<false>(sb, prm.gammavalue, prm.gamma_fast);
                const int X = ((t % tiles_x) * kTileX) / 8 + wid % wpr;
                const int Y = ((t / tiles_x) * tile_y) / 8 + (rgrp >> 1);
                if (X < prm.out_nx && Y < prm.out_ny)
                    __stcs(prm.out + o * rec + (int64_t)Y * prm.out_nx + X, sb);
            }
        } else {
            tile[ty * 33 + tx] = val;
            __syncthreads();
            const int nbx = kTileX / b, nby = tile_y / b;
            if (tx < nbx && ty < nby) {
                float s = 0.0f;                                              // :636 sum()
                for (int jj = 0; jj < b; ++jj)
                    for (int ii = 0; ii < b; ++ii) s = s + tile[(ty * b + jj) * 33 + tx * b + ii];
                s = s * prm.bindx;                                           // :640
                if (prm.mode == EBSD_SCALING_GAM)
                    s = gamma_pow<STRICT>(s, prm.gammavalue, prm.gamma_fast);
                const int X = ((t % tiles_x) * kTileX) / b + tx;
                const int Y = ((t / tiles_x) * tile_y) / b + ty;
                if (X < prm.out_nx && Y < prm.out_ny)
                    __stcs(prm.out + o * rec + (int64_t)Y * prm.out_nx + X, s);
            }
            __syncthreads();
        }
    }
}

// Orientations per CTA when the caller leaves the choice to the library:
// kAutoOpc (each CTA's per-pixel tables are reused over more orientations;
// at 640x480 262 k patterns/s with 64, 259 k with 32, 245 k with 8), halved
// while the grid would have fewer than kAutoMinCtasPerSm CTAs per SM.
constexpr int kAutoOpc = 64, kAutoMinCtasPerSm = 32;

int resolve_opc(int opc, int64_t n, int ntiles)
{
    if (opc > 0) return opc;
    // SM count of the current device, looked up once per device (a benign
    // race: every thread that looks it up stores the same value)
    constexpr int kMaxDevices = 64;
    static int sms_of[kMaxDevices] = {};
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    if (dev >= 0 && dev < kMaxDevices) sms = sms_of[dev];
    if (sms == 0) {
        if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
            sms < 1) {
            cudaGetLastError();
            sms = 1;
        }
        if (dev >= 0 && dev < kMaxDevices) sms_of[dev] = sms;
    }
    int o = kAutoOpc;
    while (o > 1 && ((n + o - 1) / o) * (int64_t)ntiles < (int64_t)kAutoMinCtasPerSm * sms) o >>= 1;
    return o;
}

// Launch bounds: CTAs of up to 512 threads (tile_y 16).  A build may trade
// the largest tile for a register budget with more resident CTAs
// (EBSD_FWD_MAX_THREADS and EBSD_FWD_MIN_BLOCKS).
#ifdef EBSD_FWD_MIN_BLOCKS
#define EBSD_FWD_LAUNCH_BOUNDS __launch_bounds__(EBSD_FWD_MAX_THREADS, EBSD_FWD_MIN_BLOCKS)
#else
#define EBSD_FWD_LAUNCH_BOUNDS __launch_bounds__(512)
#endif

template <int NV, bool STRICT, bool NOISE, bool BIN8, bool CELLS = false, bool G64 = false>
__global__ void EBSD_FWD_LAUNCH_BOUNDS k_forward(const FwdParams prm, int tile_y, int tiles_x,
                                                 int ntiles, int opc, int warp_w)
{
    extern __shared__ float tile[];  // [tile_y][33], binning only
    const int t = (int)(blockIdx.x % (unsigned)ntiles);
    const int64_t o_begin = (int64_t)(blockIdx.x / (unsigned)ntiles) * opc;
    forward_tile<NV, STRICT, NOISE, BIN8, CELLS, G64>(prm, tile_y, tiles_x, t, o_begin, opc, tile,
                                                      warp_w);
}

// Batched pattern loop: one persistent grid works through a queue of work
// items (job, tile, run of orientations) spanning jobs of different
// detectors, binnings and masters.  Each CTA takes the next item with one
// atomic increment and stops when the queue is exhausted -- no CTA waits
// on another, so nothing can spin.  Jobs are ordered by item_begin.
// The jobs' parameters are kernel parameters (a __grid_constant__ table in
// the constant bank): the pattern loop reads them through the constant
// cache as the per-job kernel does, not from shared memory, which shares
// the L1 data pipe with the master gathers (parameters staged in shared
// memory cost about ten shared loads per warp and orientation).
// TY is the tile height (CTA = 32 x TY threads: 4, 8 or 16, the job's tuned
// tile height); a group's jobs all use it, and BIN8 (the 8x8-binned
// variant of forward_tile).  CTAs get 64 registers (1024 threads per SM):
// the parameters read in the loop need registers of their own.  Every job
// of the 64-job workload through the queue, patterns/s: 282.0 k at 64
// registers, 280.5 k with nine 32 x 4 CTAs per SM (56), 273.0 k with ten 32 x
// 4 and five 32 x 8 (48, spilling); with the parameters staged in shared
// memory instead, 272.3 k (56 / 64 registers) and 276.2 k (48).
#ifndef EBSD_BATCH_MIN_BLOCKS4
#define EBSD_BATCH_MIN_BLOCKS4 8
#endif
#ifndef EBSD_BATCH_MIN_BLOCKS8
#define EBSD_BATCH_MIN_BLOCKS8 4
#endif
template <int NV, bool NOISE, int TY, bool BIN8>
__global__ void __launch_bounds__(32 * TY,
                                  TY == 4 ? (NOISE ? 8 : EBSD_BATCH_MIN_BLOCKS4)
                                  : TY == 8 ? (NOISE ? 4 : EBSD_BATCH_MIN_BLOCKS8)
                                            : 32 / TY)
    k_forward_batched(const __grid_constant__ BatchLaunch L,
                      unsigned long long* __restrict__ counter)
{
    __shared__ float tile[TY * 33];
    __shared__ long long s_obegin[2];
    __shared__ int s_job[2], s_tile[2];
    const int njobs = L.njobs;
    const long long total = L.total_items;
    // Thread 0 claims and decodes items one ahead: while the CTA computes
    // item k, the claim, the job search and the (64-bit) tile/orientation
    // split of item k+1 are already done by one thread instead of all.
    auto claim = [&](int slot) {
        const long long it = (long long)atomicAdd(counter, 1ULL);
        if (it >= total) {
            s_job[slot] = -1;
            return;
        }
        int lo = 0, hi = njobs - 1;  // last job with item_begin <= it
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (L.job[mid].item_begin <= it)
                lo = mid;
            else
                hi = mid - 1;
        }
        const BatchJob& J = L.job[lo];
        const long long local = it - J.item_begin;
        const long long ob = local / J.ntiles;
        s_job[slot] = lo;
        s_tile[slot] = (int)(local - ob * J.ntiles);
        s_obegin[slot] = ob * J.opc;
    };
    if (threadIdx.x == 0) claim(0);
    __syncthreads();
    // One barrier per item: the next item's slot is written by thread 0
    // while the others read this one's, and the barrier at the end of the
    // item publishes it (it also keeps the CTA's warps on one item, whose
    // gathers share L1 lines).
    for (int slot = 0;; slot ^= 1) {
        const int job = s_job[slot];
        if (job < 0) break;
        const int t = s_tile[slot];
        const int64_t o_begin = s_obegin[slot];
        if (threadIdx.x == 0) claim(slot ^ 1);
        const BatchJob& J = L.job[job];
        forward_tile<NV, false, NOISE, BIN8>(J.p, TY, J.tiles_x, t, o_begin, J.opc, tile, 16);
        __syncthreads();
    }
}

template <int NV, bool STRICT, bool NOISE, bool BIN8 = false, bool CELLS = false,
          bool G64 = false>
cudaError_t launch_nv2(const FwdParams& p, const LaunchCfg& cfg, cudaStream_t s)
{
    // binned records are summed inside a CTA: its height must hold whole
    // b x b blocks (binning 8 on a 4-row tile would write nothing)
    int tile_y = cfg.tile_y;
    if (p.mode != EBSD_SCALING_NOT && p.binning > 1)
        while (tile_y % p.binning != 0 && tile_y < 16) tile_y *= 2;
    const int tiles_x = (p.numsx + kTileX - 1) / kTileX;
    const int tiles_y = (p.numsy + tile_y - 1) / tile_y;
    const int ntiles = tiles_x * tiles_y;
    const int opc = resolve_opc(cfg.orient_per_cta, p.n, ntiles);
    const int64_t oblocks = (p.n + opc - 1) / opc;
    const int64_t blocks = oblocks * ntiles;
    if (blocks > 0x7fffffffLL) return cudaErrorInvalidConfiguration;
    cudaLaunchConfig_t lc = {};
    lc.gridDim = dim3((unsigned)blocks);
    lc.blockDim = dim3(kTileX * tile_y);
    lc.dynamicSmemBytes = sizeof(float) * 33 * tile_y;
    lc.stream = s;
    cudaLaunchAttribute attr[1];
    set_persist_attr(cfg, attr, lc);
    const int warp_w = cfg.warp_w == 32 ? 32 : 16;
    return cudaLaunchKernelEx(&lc, k_forward<NV, STRICT, NOISE, BIN8, CELLS, G64>, p, tile_y,
                              tiles_x, ntiles, opc, warp_w);
}

template <int NV>
cudaError_t launch_nv(const FwdParams& p, const LaunchCfg& cfg, cudaStream_t s, bool cells)
{
    const bool bin8 = !cfg.strict && p.mode != EBSD_SCALING_NOT && p.binning == 8;
    if (p.accurate == 2) {  // binary64 geometry (fused gather; no cells variant; <= 32 bins)
        if constexpr (NV <= 8) {
            if (cells || !p.rg64) return cudaErrorInvalidValue;
            const bool b8 = p.mode != EBSD_SCALING_NOT && p.binning == 8;
            if (p.poisson)
                return b8 ? launch_nv2<NV, false, true, true, false, true>(p, cfg, s)
                          : launch_nv2<NV, false, true, false, false, true>(p, cfg, s);
            return b8 ? launch_nv2<NV, false, false, true, false, true>(p, cfg, s)
                      : launch_nv2<NV, false, false, false, false, true>(p, cfg, s);
        }
        return cudaErrorInvalidValue;
    }
    if (cells)  // the diagnostic instantiations (no noise)
        return cfg.strict ? launch_nv2<NV, true, false, false, true>(p, cfg, s)
               : bin8     ? launch_nv2<NV, false, false, true, true>(p, cfg, s)
                          : launch_nv2<NV, false, false, false, true>(p, cfg, s);
    if (p.poisson)  // noise: fused gather
        return bin8 ? launch_nv2<NV, false, true, true>(p, cfg, s)
                    : launch_nv2<NV, false, true>(p, cfg, s);
    if (cfg.strict) return launch_nv2<NV, true, false>(p, cfg, s);
    return bin8 ? launch_nv2<NV, false, false, true>(p, cfg, s)
                : launch_nv2<NV, false, false>(p, cfg, s);
}

template <int NV, bool NOISE, int TY, bool BIN8>
cudaError_t launch_batched3(const BatchLaunch& L, unsigned long long* counter, int grid,
                            cudaStream_t s)
{
    k_forward_batched<NV, NOISE, TY, BIN8><<<grid, 32 * TY, 0, s>>>(L, counter);
    return cudaGetLastError();
}

// The group shapes: (TY, BIN8) in {(4, no), (8, no), (8, yes), (16, no), (16, yes)}.
template <int NV, bool NOISE>
cudaError_t launch_batched_nv2(const BatchLaunch& L, unsigned long long* counter, int grid,
                               int ty, bool bin8, cudaStream_t s)
{
    if (ty == 4 && !bin8) return launch_batched3<NV, NOISE, 4, false>(L, counter, grid, s);
    if (ty == 8)
        return bin8 ? launch_batched3<NV, NOISE, 8, true>(L, counter, grid, s)
                    : launch_batched3<NV, NOISE, 8, false>(L, counter, grid, s);
    if (ty == 16)
        return bin8 ? launch_batched3<NV, NOISE, 16, true>(L, counter, grid, s)
                    : launch_batched3<NV, NOISE, 16, false>(L, counter, grid, s);
    return cudaErrorInvalidValue;
}

template <int NV>
cudaError_t launch_batched_nv(const BatchLaunch& L, unsigned long long* counter, int grid,
                              bool noise, int ty, bool bin8, cudaStream_t s)
{
    return noise ? launch_batched_nv2<NV, true>(L, counter, grid, ty, bin8, s)
                 : launch_batched_nv2<NV, false>(L, counter, grid, ty, bin8, s);
}

template <int NV, bool NOISE, int TY, bool BIN8>
int batched_grid3()
{
    int dev = 0, sms = 0, per = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_forward_batched<NV, NOISE, TY, BIN8>,
                                                  32 * TY, 0);
    return sms * (per > 0 ? per : 1);
}

template <int NV, bool NOISE>
int batched_grid_nv2(int ty, bool bin8)
{
    if (ty == 4 && !bin8) return batched_grid3<NV, NOISE, 4, false>();
    if (ty == 8) return bin8 ? batched_grid3<NV, NOISE, 8, true>() : batched_grid3<NV, NOISE, 8, false>();
    if (ty == 16)
        return bin8 ? batched_grid3<NV, NOISE, 16, true>() : batched_grid3<NV, NOISE, 16, false>();
    return 0;
}

template <int NV>
int batched_grid_nv(bool noise, int ty, bool bin8)
{
    return noise ? batched_grid_nv2<NV, true>(ty, bin8) : batched_grid_nv2<NV, false>(ty, bin8);
}

}  // namespace

cudaError_t launch_forward_batched(const BatchLaunch& L, unsigned long long* counter, int NV,
                                   bool noise, int ty, bool bin8, int grid, cudaStream_t s)
{
    if (!batch_shape_ok(ty, bin8) || L.njobs < 1 || L.njobs > kBatchLaunchJobs)
        return cudaErrorInvalidValue;
    switch (NV) {
        case 1: return launch_batched_nv<1>(L, counter, grid, noise, ty, bin8, s);
        case 2: return launch_batched_nv<2>(L, counter, grid, noise, ty, bin8, s);
        case 3: return launch_batched_nv<3>(L, counter, grid, noise, ty, bin8, s);
        case 4: return launch_batched_nv<4>(L, counter, grid, noise, ty, bin8, s);
        case 5: return launch_batched_nv<5>(L, counter, grid, noise, ty, bin8, s);
        case 6: return launch_batched_nv<6>(L, counter, grid, noise, ty, bin8, s);
        case 7: return launch_batched_nv<7>(L, counter, grid, noise, ty, bin8, s);
        case 8: return launch_batched_nv<8>(L, counter, grid, noise, ty, bin8, s);
        default: return cudaErrorInvalidValue;
    }
}

int batched_grid(int NV, bool noise, int ty, bool bin8)
{
    if (!batch_shape_ok(ty, bin8)) return 0;
    switch (NV) {
        case 1: return batched_grid_nv<1>(noise, ty, bin8);
        case 2: return batched_grid_nv<2>(noise, ty, bin8);
        case 3: return batched_grid_nv<3>(noise, ty, bin8);
        case 4: return batched_grid_nv<4>(noise, ty, bin8);
        case 5: return batched_grid_nv<5>(noise, ty, bin8);
        case 6: return batched_grid_nv<6>(noise, ty, bin8);
        case 7: return batched_grid_nv<7>(noise, ty, bin8);
        case 8: return batched_grid_nv<8>(noise, ty, bin8);
        default: return 0;
    }
}

int64_t forward_ctas(const FwdParams& p, const LaunchCfg& cfg)
{
    int tile_y = cfg.tile_y;
    if (p.mode != EBSD_SCALING_NOT && p.binning > 1)
        while (tile_y % p.binning != 0 && tile_y < 16) tile_y *= 2;
    const int ntiles = ((p.numsx + kTileX - 1) / kTileX) * ((p.numsy + tile_y - 1) / tile_y);
    const int opc = resolve_opc(cfg.orient_per_cta, p.n, ntiles);
    return ((p.n + opc - 1) / opc) * (int64_t)ntiles;
}

cudaError_t launch_forward(const FwdParams& p, int NV, const LaunchCfg& cfg, cudaStream_t s,
                           bool cells)
{
    if (p.n <= 0) return cudaSuccess;
    if (cells && (!p.nix || !p.niy || !p.ixy0 || !p.ixy1)) return cudaErrorInvalidValue;
    switch (NV) {
        case 1: return launch_nv<1>(p, cfg, s, cells);
        case 2: return launch_nv<2>(p, cfg, s, cells);
        case 3: return launch_nv<3>(p, cfg, s, cells);
        case 4: return launch_nv<4>(p, cfg, s, cells);
        case 5: return launch_nv<5>(p, cfg, s, cells);
        case 6: return launch_nv<6>(p, cfg, s, cells);
        case 7: return launch_nv<7>(p, cfg, s, cells);
        case 8: return launch_nv<8>(p, cfg, s, cells);
        case 9: return launch_nv<9>(p, cfg, s, cells);
        case 10: return launch_nv<10>(p, cfg, s, cells);
        case 11: return launch_nv<11>(p, cfg, s, cells);
        case 12: return launch_nv<12>(p, cfg, s, cells);
        case 13: return launch_nv<13>(p, cfg, s, cells);
        case 14: return launch_nv<14>(p, cfg, s, cells);
        case 15: return launch_nv<15>(p, cfg, s, cells);
        case 16: return launch_nv<16>(p, cfg, s, cells);
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace ebsd
