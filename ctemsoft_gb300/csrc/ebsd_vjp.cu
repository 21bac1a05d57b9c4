// Adjoint of the EBSD pattern loop: vector-Jacobian products of the output
// records with respect to the left rotation tangent (w0, w1, w2) of each
// orientation, q(w) = exp(w) (x) q, and the pattern centre (xpc, ypc, L).
//
// The forward gather is recomputed, never stored.  Per pixel the kernel
// evaluates P = pref * sum_k W_k B_k and its six partial derivatives J_p:
//   * through the bilinear fractions of the master gather (the cell index
//     is locally constant), the square-Lambert Jacobian, the normalisation
//     and fold of the rotated direction d = q (x) rg (x) conj(q):
//     dP/dw = d x g_d, g_d = dP/dd;
//   * through the detector direction rg (dP/dtheta = (M^T g_d) . drg/dtheta)
//     and the Monte-Carlo weights (sum_k dW_k/dtheta B_k), both from
//     binary64 derivative tables built at detector set-up.
// The pixel sums needed by each mode are reduced per CTA with warp
// shuffles into a scratch buffer of partials, which a second kernel sums
// per orientation in binary64 in a fixed order (deterministic results).
//
// Modes: EBSD_VJP_COTANGENT, grad = sum_B cot(B) dO(B)/dphi; EBSD_VJP_NDP,
// the loss 1 - <O,T>/(|O||T|) against target records T and its gradient,
// from one pass: sum T J, sum O J and the three dot products.
#include "ebsd_device.cuh"
#include "ebsd_internal.h"

namespace ebsd {

namespace {

// Sum each of KP per-lane values over the warp (reduce-scatter butterfly:
// every step halves the values a lane carries, so KP values cost about KP
// shuffles instead of 5 KP).  On return lane l holds the warp total of value
// index l / (32 / KP) in v[0].
template <int KP>
__device__ __forceinline__ void warp_reduce_scatter(float (&v)[KP], int lane)
{
    int off = 16;
#pragma unroll
    for (int n = KP; n > 1; n >>= 1, off >>= 1) {
        const bool upper = (lane & off) != 0;
#pragma unroll
        for (int i = 0; i < n / 2; ++i) {
            const float send = upper ? v[i] : v[i + n / 2];
            const float keep = upper ? v[i + n / 2] : v[i];
            v[i] = keep + __shfl_xor_sync(0xffffffffu, send, off);
        }
    }
#pragma unroll
    for (; off > 0; off >>= 1) v[0] += __shfl_xor_sync(0xffffffffu, v[0], off);
}

// Pixel (tx, ty) of thread tid in a 32-wide tile.  BSH (binning 2 or 4):
// each warp covers a 32/b x b block, so every binning block lies within one
// warp and is summed with shuffles (adj_block_sum); otherwise warps are rows.
// The kernels take BSH as a template argument, so that the unbinned variant
// carries none of it (a runtime test cost 3 % at 640x480).
template <bool BSH>
__device__ __forceinline__ void adj_pixel(int tid, int b, int& tx, int& ty)
{
    const int lane = tid & 31, wid = tid >> 5;
    if (BSH) {
        const int bw = 32 / b;  // warps per tile row: kTileX / bw = b
        tx = (wid % b) * bw + lane % bw;
        ty = (wid / b) * b + lane / bw;
    } else {
        tx = lane;
        ty = wid;
    }
}

// Sum of v over the b x b binning block that holds this lane (b = 2 or 4,
// warp = 32/b x b lanes, row-major); every lane of the block gets the total.
__device__ __forceinline__ float adj_block_sum(float v, int b)
{
    const int bw = 32 / b;
    for (int m = 1; m < b; m <<= 1) v += __shfl_xor_sync(0xffffffffu, v, m);
    for (int m = 1; m < b; m <<= 1) v += __shfl_xor_sync(0xffffffffu, v, m * bw);
    return v;
}

// Per-orientation geometry of one pixel for the adjoint: the rotated
// direction d, its normalised and folded h (fold sign s, 1/|d| ind), the
// Lambert point's Jacobian rows dX, dY, and the cell and bilinear fractions.
struct AdjGeom {
    float d0, d1, d2, h0, h1, h2, s, ind;
    float dX[3], dY[3];
    int ix0, iy0;
    float dx, dy;
};

__device__ __forceinline__ void adj_geometry(const FwdParams& prm, const float4 q, const float4 r,
                                             AdjGeom& g)
{
    rotate_direction(q, r.x, r.y, r.z, g.d0, g.d1, g.d2);
    // normalisation and fold (:588-589) with the hardware reciprocal square
    // root: the adjoint needs relative accuracy, not the reference's rounding
    g.ind = rsqrtf(fmaf(g.d0, g.d0, fmaf(g.d1, g.d1, g.d2 * g.d2)));
    g.h0 = g.d0 * g.ind;
    g.h1 = g.d1 * g.ind;
    g.h2 = g.d2 * g.ind;
    g.s = g.h2 < 0.0f ? -1.0f : 1.0f;
    float LX, LY;
    lambert_inverse_jac(g.s * g.h0, g.s * g.h1, g.s * g.h2, prm.spi2, LX, LY, g.dX, g.dY);
    int nix, niy;
    g.ix0 = lambert_cell(prm.scl * LX, prm.npx, g.dx, nix);
    g.iy0 = lambert_cell(prm.scl * LY, prm.npy, g.dy, niy);
}

// The four weighted corner sums SA = sum_k W_k A_k ... SD of the gather and
// the weight-slope sums U0 = sum_k G0_k bv_k, U1 = sum_k G1_k bv_k (bv_k the
// per-bin bilinear value): S = (SA, SB, SC, SD, U0, U1).  P and both
// bilinear slopes follow from SA..SD with four FMAs per bin, and since
// dW_k/dtheta_a = G0_k di0_a + G1_k di1_a the weight terms need only U0, U1.
// The sums run on packed pairs of bins (even bins in the low halves, odd in
// the high), two fused multiply-adds per instruction.
template <int NV>
__device__ __forceinline__ void adj_gather(const FwdParams& prm, const VjpParams& vp, int p,
                                           uint64_t pol, const AdjGeom& g, float (&S)[6])
{
    const int ix1 = min(g.ix0 + 1, 2 * prm.npx), iy1 = min(g.iy0 + 1, 2 * prm.npy);
    // node offsets in 32 bits: ebsd_set_master keeps the master below 2^31 float4
    const float4* m00 = prm.master + (uint32_t)(g.iy0 * prm.gx + g.ix0) * (uint32_t)NV;
    const int col = (ix1 - g.ix0) * NV;             // 0 at the grid's last column
    const int row = (iy1 - g.iy0) * prm.gx * NV;    // 0 at its last row
    const float dxm = 1.0f - g.dx, dym = 1.0f - g.dy;
    const float w00 = dxm * dym, w10 = g.dx * dym, w01 = dxm * g.dy, w11 = g.dx * g.dy;
    const f2_t W00 = f2_pack(w00, w00), W10 = f2_pack(w10, w10), W01 = f2_pack(w01, w01),
               W11 = f2_pack(w11, w11);
    f2_t acc[6] = {0, 0, 0, 0, 0, 0};  // +0.0f pairs
    const float4* wp = prm.W + p;      // plane c of W at wp + c P
    const float4* ep = vp.dW + p;      // plane c of G0; G1 NV planes further
    const int64_t plane = prm.P, eplane = (int64_t)NV * prm.P;
    // one float4 group of bins at a time: unrolling would hoist all the
    // vector loads and spill
#pragma unroll 1
    for (int c = 0; c < NV; ++c, wp += plane, ep += plane) {
        f2_t A[2], B[2], C[2], D[2], wc[2], e0[2], e1[2];
        const float4* m = m00 + c;
        ldg4_keep2(m, pol, A[0], A[1]);
        ldg4_keep2(m + col, pol, B[0], B[1]);
        ldg4_keep2(m + row, pol, C[0], C[1]);
        ldg4_keep2(m + row + col, pol, D[0], D[1]);
        ldg4_keep2(wp, pol, wc[0], wc[1]);
        ldg4_keep2(ep, pol, e0[0], e0[1]);
        ldg4_keep2(ep + eplane, pol, e1[0], e1[1]);
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const f2_t bv = f2_fma(A[h], W00, f2_fma(B[h], W10, f2_fma(C[h], W01, f2_mul(D[h], W11))));
            acc[0] = f2_fma(wc[h], A[h], acc[0]);
            acc[1] = f2_fma(wc[h], B[h], acc[1]);
            acc[2] = f2_fma(wc[h], C[h], acc[2]);
            acc[3] = f2_fma(wc[h], D[h], acc[3]);
            acc[4] = f2_fma(e0[h], bv, acc[4]);
            acc[5] = f2_fma(e1[h], bv, acc[5]);
        }
    }
#pragma unroll
    for (int i = 0; i < 6; ++i) S[i] = f2_sum(acc[i]);
}

// Value and the six derivatives of one orientation from its geometry and
// gather sums; t0..t2 are the drg planes (d rg/d(xpc, ypc, L), with d Dx/d
// theta in .w) and di1 the plane of d Dy/d theta.
__device__ __forceinline__ void adj_finish(const FwdParams& prm, const float4 q, const AdjGeom& g,
                                           const float (&S)[6], const float4 t0, const float4 t1,
                                           const float4 t2, const float4 di1, float pref,
                                           float& val, float (&J)[6])
{
    const float SA = S[0], SB = S[1], SC = S[2], SD = S[3], U0 = S[4], U1 = S[5];
    const float dxm = 1.0f - g.dx, dym = 1.0f - g.dy;
    const float w00 = dxm * dym, w10 = g.dx * dym, w01 = dxm * g.dy, w11 = g.dx * g.dy;
    const float P = fmaf(SA, w00, fmaf(SB, w10, fmaf(SC, w01, SD * w11)));
    const float gX = fmaf(SB - SA, dym, (SD - SC) * g.dy);
    const float gY = fmaf(SC - SA, dxm, (SD - SB) * g.dx);
    val = pref * P;
    const float sx = prm.scl * pref * gX, sy = prm.scl * pref * gY;
    const float gc0 = sx * g.dX[0] + sy * g.dY[0];
    const float gc1 = sx * g.dX[1] + sy * g.dY[1];
    const float gc2 = sx * g.dX[2] + sy * g.dY[2];
    const float pr = gc0 * g.h0 + gc1 * g.h1 + gc2 * g.h2;
    const float k = g.s * g.ind;
    const float g0 = k * (gc0 - pr * g.h0), g1 = k * (gc1 - pr * g.h1), g2 = k * (gc2 - pr * g.h2);
    J[0] = g.d1 * g2 - g.d2 * g1;
    J[1] = g.d2 * g0 - g.d0 * g2;
    J[2] = g.d0 * g1 - g.d1 * g0;
    // M^T g = conj(q) (x) (0,g) (x) q
    const float u0 = -(g0 * q.y) - g1 * q.z - g2 * q.w;
    const float u1 = g0 * q.x + g1 * q.w - g2 * q.z;
    const float u2 = -(g0 * q.w) + g1 * q.x + g2 * q.y;
    const float u3 = g0 * q.z - g1 * q.y + g2 * q.x;
    const float m0 = q.x * u1 - q.y * u0 - q.z * u3 + q.w * u2;
    const float m1 = q.x * u2 + q.y * u3 - q.z * u0 - q.w * u1;
    const float m2 = q.x * u3 - q.y * u2 + q.z * u1 - q.w * u0;
    J[3] = m0 * t0.x + m1 * t0.y + m2 * t0.z + pref * fmaf(U0, t0.w, U1 * di1.x);
    J[4] = m0 * t1.x + m1 * t1.y + m2 * t1.z + pref * fmaf(U0, t1.w, U1 * di1.y);
    J[5] = m0 * t2.x + m1 * t2.y + m2 * t2.z + pref * fmaf(U0, t2.w, U1 * di1.z);
}

// Value and the six derivatives (w0, w1, w2, xpc, ypc, L) of output pixel p
// of orientation o, before binning.
template <int NV>
__device__ __forceinline__ void pixel_value_jacobian(const FwdParams& prm, const VjpParams& vp,
                                                     int p, int64_t o, uint64_t pol,
                                                     float pref, float& val, float (&J)[6])
{
    const float4 q = __ldg(prm.quats + o);
    const float4 r = ldg4_keep(prm.rg + p, pol);
    AdjGeom g;
    adj_geometry(prm, q, r, g);
    float S[6];
    adj_gather<NV>(prm, vp, p, pol, g, S);
    const int64_t eplane = (int64_t)NV * prm.P;
    const float4 t0 = ldg4_keep(vp.drg + p, pol), t1 = ldg4_keep(vp.drg + prm.P + p, pol),
                 t2 = ldg4_keep(vp.drg + 2 * (int64_t)prm.P + p, pol);
    const float4 di1 = ldg4_keep(vp.dW + 2 * eplane + p, pol);  // (xpc, ypc, L)
    adj_finish(prm, q, g, S, t0, t1, t2, di1, pref, val, J);
}

// Resident CTAs per SM the register allocation is held to (256 threads
// each); a build-time tuning knob.  3 (80 registers: 6 CTAs of 32 x 4
// pixels per SM) measured 1.5 % faster at 640x480 than 4 (64 registers,
// which spills).
#ifndef EBSD_VJP_MIN_BLOCKS
#define EBSD_VJP_MIN_BLOCKS 3
#endif

template <int NV, int MODE, bool BSH>
__global__ void __launch_bounds__(256, EBSD_VJP_MIN_BLOCKS)
    k_vjp(const FwdParams prm, const VjpParams vp, int tile_y, int tiles_x, int ntiles, int opc)
{
    constexpr int K = MODE == EBSD_VJP_NDP ? 15 : 6;
    constexpr int KP = MODE == EBSD_VJP_NDP ? 16 : 8;
    // [tile_y][33] pattern tile, then [opc][tile_y][K] warp sums
    extern __shared__ float sm[];
    float* tile = sm;
    float* red = sm + 33 * tile_y;
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    int tx, ty;
    adj_pixel<BSH>(tid, vp.binning, tx, ty);
    // Orientation blocks vary fastest across the grid: the CTAs resident at
    // any moment cover a few tiles for many orientations, so each tile's
    // per-pixel tables (W, dW, rg, drg: larger than L2 together with the
    // master at 640x480) are read from DRAM about once, not once per sweep.
    const unsigned n_ob = (unsigned)((prm.n + opc - 1) / opc);
    const int t = (int)(blockIdx.x / n_ob);
    const int64_t o_begin = (int64_t)(blockIdx.x % n_ob) * opc;
    const int x = (t % tiles_x) * kTileX + tx;
    const int y = (t / tiles_x) * tile_y + ty;
    const int b = vp.binning;
    // only pixels of full output blocks contribute (binning crops to the floor)
    const bool inside = x < prm.numsx && y < prm.numsy && x < prm.out_nx * b &&
                        y < prm.out_ny * b;
    const int p = y * prm.numsx + x;
    // per-pixel constants (direction, weights and their derivative tables)
    // are re-read per orientation; they are L1/L2 hits, and keeping them out
    // of registers lets 3 CTAs share an SM without spilling
    const uint64_t pol = l2_policy_evict_last();
    const float pref = (float)prm.prefactor;
    const float ib2 = 1.0f / (float)(b * b);
    const int64_t rec = (int64_t)prm.out_nx * prm.out_ny;
    const int X = x / b, Y = y / b;
    const bool leader = (x % b == 0) && (y % b == 0);

    for (int64_t o = o_begin; o < o_begin + opc && o < prm.n; ++o) {
        float val = 0.0f, J[6] = {0, 0, 0, 0, 0, 0};
        if (inside) pixel_value_jacobian<NV>(prm, vp, p, o, pol, pref, val, J);
        // output-record value of this pixel's block
        float O = val;
        if (BSH) {
            O = adj_block_sum(val, b) * ib2;
        } else if (b > 1) {
            tile[ty * 33 + tx] = val;
            __syncthreads();
            if (inside) {
                const int bx = tx - tx % b, by = ty - ty % b;
                float s2 = 0.0f;
                for (int jj = 0; jj < b; ++jj)
                    for (int ii = 0; ii < b; ++ii) s2 += tile[(by + jj) * 33 + bx + ii];
                O = s2 * ib2;
            }
            __syncthreads();
        }
        float acc[KP];
#pragma unroll
        for (int a = K; a < KP; ++a) acc[a] = 0.0f;
        if (inside) {
            const float dv = vp.data[o * rec + (int64_t)Y * prm.out_nx + X];
            if (MODE == EBSD_VJP_NDP) {
                const float cT = dv * ib2, cO = O * ib2;
#pragma unroll
                for (int a = 0; a < 6; ++a) {
                    acc[a] = cT * J[a];
                    acc[6 + a] = cO * J[a];
                }
                acc[12] = leader ? O * O : 0.0f;
                acc[13] = leader ? O * dv : 0.0f;
                acc[14] = leader ? dv * dv : 0.0f;
            } else {
                const float c = dv * ib2;
#pragma unroll
                for (int a = 0; a < 6; ++a) acc[a] = c * J[a];
            }
        } else {
#pragma unroll
            for (int a = 0; a < K; ++a) acc[a] = 0.0f;
        }
        warp_reduce_scatter<KP>(acc, lane);
        {
            // each warp its own slot per orientation: no barrier until the end
            const int idx = lane / (32 / KP);
            if (lane % (32 / KP) == 0 && idx < K) red[((o - o_begin) * tile_y + wid) * K + idx] = acc[0];
        }
    }
    __syncthreads();
    const int no = (int)min((int64_t)opc, prm.n - o_begin);
    for (int i = tid; i < no * K; i += blockDim.x) {
        const int ol = i / K, k = i - ol * K;
        float s2 = 0.0f;
        for (int wy = 0; wy < tile_y; ++wy) s2 += red[(ol * tile_y + wy) * K + k];
        vp.partial[((o_begin + ol) * ntiles + t) * K + k] = s2;
    }
}

// The adjoint for unbinned records: CTAs of four warps over a 32 x 4 PPT
// pixel tile, each thread PPT pixels (rows ty, ty + 4, ...) of the tile.  A
// thread adds its pixels' terms before the warp reduction, so the
// reduction (about 85 instructions per warp-orientation) is paid once per
// PPT pixels.  Each warp covers a 16 x 2 block of every 32 x 4 layer of
// the tile in 4 x 2 quarter-warps, so that the 8 lanes whose 128-bit loads
// the L1 serves together gather from a compact patch of the master.
// Resident CTAs per SM for its register budget (a build-time knob): 5 (96
// registers) measured 4-5 % faster at 640x480 and 480x480 than 6 (80,
// where the loss mode spills at four pixels per thread) and 12 % faster
// than 8 (64).
#ifndef EBSD_VJP1_MIN_BLOCKS
#define EBSD_VJP1_MIN_BLOCKS 5
#endif
template <int NV, int MODE, int PPT>
__global__ void __launch_bounds__(128, EBSD_VJP1_MIN_BLOCKS)
    k_vjp1(const FwdParams prm, const VjpParams vp, int tiles_x, int ntiles, int opc)
{
    constexpr int K = MODE == EBSD_VJP_NDP ? 15 : 6;
    constexpr int KP = MODE == EBSD_VJP_NDP ? 16 : 8;
    extern __shared__ float red[];  // [opc][4 warps][K] warp sums
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const int tx = (wid & 1) * 16 + (lane >> 3) * 4 + (lane & 3);
    const int ty = (wid >> 1) * 2 + ((lane >> 2) & 1);
    // orientation blocks fastest across the grid (as k_vjp)
    const unsigned n_ob = (unsigned)((prm.n + opc - 1) / opc);
    const int t = (int)(blockIdx.x / n_ob);
    const int64_t o_begin = (int64_t)(blockIdx.x % n_ob) * opc;
    const int x = (t % tiles_x) * kTileX + tx;
    const int y0 = (t / tiles_x) * (4 * PPT) + ty;
    const uint64_t pol = l2_policy_evict_last();
    const float pref = (float)prm.prefactor;
    const int64_t rec = (int64_t)prm.P;  // unbinned: out_nx x out_ny = numsx x numsy

    for (int64_t o = o_begin; o < o_begin + opc && o < prm.n; ++o) {
        float acc[KP];
#pragma unroll
        for (int a = 0; a < KP; ++a) acc[a] = 0.0f;
#pragma unroll
        for (int k = 0; k < PPT; ++k) {
            const int y = y0 + 4 * k;
            if (x < prm.numsx && y < prm.numsy) {
                const int p = y * prm.numsx + x;
                float val, J[6];
                pixel_value_jacobian<NV>(prm, vp, p, o, pol, pref, val, J);
                const float dv = vp.data[o * rec + p];
#pragma unroll
                for (int a = 0; a < 6; ++a) acc[a] = fmaf(dv, J[a], acc[a]);
                if (MODE == EBSD_VJP_NDP) {
#pragma unroll
                    for (int a = 0; a < 6; ++a) acc[6 + a] = fmaf(val, J[a], acc[6 + a]);
                    acc[12] = fmaf(val, val, acc[12]);
                    acc[13] = fmaf(val, dv, acc[13]);
                    acc[14] = fmaf(dv, dv, acc[14]);
                }
            }
        }
        warp_reduce_scatter<KP>(acc, lane);
        const int idx = lane / (32 / KP);
        if (lane % (32 / KP) == 0 && idx < K) red[((o - o_begin) * 4 + wid) * K + idx] = acc[0];
    }
    __syncthreads();
    const int no = (int)min((int64_t)opc, prm.n - o_begin);
    for (int i = tid; i < no * K; i += blockDim.x) {
        const int ol = i / K, k = i - ol * K;
        float s2 = 0.0f;
        for (int w = 0; w < 4; ++w) s2 += red[(ol * 4 + w) * K + k];
        vp.partial[((o_begin + ol) * ntiles + t) * K + k] = s2;
    }
}

// Sum the per-CTA partials of each orientation in binary64 and form the
// outputs.  One warp per orientation; lanes stride over tiles in a fixed
// order, then a fixed-order shuffle tree.
template <int MODE>
__global__ void k_vjp_reduce(const float* __restrict__ partial, int64_t n, int ntiles,
                             float* __restrict__ loss, float* __restrict__ grad)
{
    constexpr int K = MODE == EBSD_VJP_NDP ? 15 : 6;
    const int64_t o = (int64_t)blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (o >= n) return;
    double s[K];
#pragma unroll
    for (int a = 0; a < K; ++a) s[a] = 0.0;
    for (int t = lane; t < ntiles; t += 32) {
        const float* pp = partial + ((int64_t)o * ntiles + t) * K;
#pragma unroll
        for (int a = 0; a < K; ++a) s[a] += (double)pp[a];
    }
#pragma unroll
    for (int a = 0; a < K; ++a)
        for (int off = 16; off > 0; off >>= 1) s[a] += __shfl_xor_sync(0xffffffffu, s[a], off);
    if (lane != 0) return;
    const int64_t og = o;
    if (MODE == EBSD_VJP_NDP) {
        const double soo = s[12], sot = s[13], stt = s[14];
        const double den = sqrt(soo * stt);
        const bool ok = den > 0.0;
        if (loss) loss[og] = ok ? (float)(1.0 - sot / den) : 0.0f;
        for (int a = 0; a < 6; ++a)
            grad[og * 6 + a] = ok ? (float)(-(s[a] - sot / soo * s[6 + a]) / den) : 0.0f;
    } else {
        if (loss) loss[og] = 0.0f;
        for (int a = 0; a < 6; ++a) grad[og * 6 + a] = (float)s[a];
    }
}

// ----------------------------------------------------------------------
// Gauss-Newton on the normalised residual r = O/|O| - T/|T| (|r|^2/2 =
// 1 - <O,T>/(|O||T|)).  With J_B = dO_B/dphi (6 parameters), a = sum O J/|O|:
//   H = (sum_B J_B J_B^T - a a^T) / |O|^2,
//   g = (a cos - sum_B T_B J_B / |T|) / |O|.
// One pass per pattern accumulates sum J J^T (21), sum T J, sum O J and the
// three dot products (36 numbers per CTA); J_B of a binned output pixel is
// the block sum of the pixel Jacobians over b^2.
constexpr int kGnK = 36;
constexpr int kGnSys = 28;  // per pattern: H (21, packed upper), g (6), loss

__device__ __forceinline__ int pk(int i, int j)  // packed index of H(i,j), i <= j
{
    return i * 6 - (i * (i - 1)) / 2 + (j - i);
}

template <int NV, bool BSH>
// Resident CTAs per SM for the Gauss-Newton kernel's register budget (256
// threads each): 3 gives 79 registers, no spills, and 11 % faster
// refinement than 2 (111 registers) on 120x120 (480x480 binned 4).
#ifndef EBSD_GN_MIN_BLOCKS
#define EBSD_GN_MIN_BLOCKS 3
#endif
__global__ void __launch_bounds__(256, EBSD_GN_MIN_BLOCKS) k_gn(const FwdParams prm, const VjpParams vp,
                                               int tile_y, int tiles_x, int ntiles, int opc)
{
    extern __shared__ float sm[];  // val tile, 6 J tiles, [tile_y][36] warp sums
    float* tile = sm;
    float* jt = sm + 33 * tile_y;
    float* red = jt + 6 * 33 * tile_y;
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    int tx, ty;
    adj_pixel<BSH>(tid, vp.binning, tx, ty);
    // Orientation blocks vary fastest across the grid: the CTAs resident at
    // any moment cover a few tiles for many orientations, so each tile's
    // per-pixel tables (W, dW, rg, drg: larger than L2 together with the
    // master at 640x480) are read from DRAM about once, not once per sweep.
    const unsigned n_ob = (unsigned)((prm.n + opc - 1) / opc);
    const int t = (int)(blockIdx.x / n_ob);
    const int64_t o_begin = (int64_t)(blockIdx.x % n_ob) * opc;
    const int x = (t % tiles_x) * kTileX + tx;
    const int y = (t / tiles_x) * tile_y + ty;
    const int b = vp.binning;
    const bool inside = x < prm.numsx && y < prm.numsy && x < prm.out_nx * b &&
                        y < prm.out_ny * b;
    const int p = y * prm.numsx + x;
    const uint64_t pol = l2_policy_evict_last();
    const float pref = (float)prm.prefactor;
    const float ib2 = 1.0f / (float)(b * b);
    const int64_t rec = (int64_t)prm.out_nx * prm.out_ny;
    const int X = x / b, Y = y / b;
    const bool leader = (x % b == 0) && (y % b == 0);

    for (int64_t o = o_begin; o < o_begin + opc && o < prm.n; ++o) {
        float val = 0.0f, J[6] = {0, 0, 0, 0, 0, 0};
        if (inside) pixel_value_jacobian<NV>(prm, vp, p, o, pol, pref, val, J);
        float O = val, JB[6];
#pragma unroll
        for (int a = 0; a < 6; ++a) JB[a] = J[a];
        if (BSH) {  // block sums within the warp
            O = adj_block_sum(val, b) * ib2;
#pragma unroll
            for (int a = 0; a < 6; ++a) JB[a] = adj_block_sum(J[a], b) * ib2;
        } else if (b > 1) {
            tile[ty * 33 + tx] = val;
#pragma unroll
            for (int a = 0; a < 6; ++a) jt[(a * tile_y + ty) * 33 + tx] = inside ? J[a] : 0.0f;
            __syncthreads();
            if (inside) {
                const int bx = tx - tx % b, by = ty - ty % b;
                float s2 = 0.0f;
                for (int jj = 0; jj < b; ++jj)
                    for (int ii = 0; ii < b; ++ii) s2 += tile[(by + jj) * 33 + bx + ii];
                O = s2 * ib2;
                if (leader) {
#pragma unroll
                    for (int a = 0; a < 6; ++a) {
                        float sj = 0.0f;
                        for (int jj = 0; jj < b; ++jj)
                            for (int ii = 0; ii < b; ++ii)
                                sj += jt[(a * tile_y + ty + jj) * 33 + tx + ii];
                        JB[a] = sj * ib2;
                    }
                }
            }
            __syncthreads();
        }
        float acc[16], accm[32];
#pragma unroll
        for (int a = 0; a < 16; ++a) acc[a] = 0.0f;
#pragma unroll
        for (int a = 0; a < 32; ++a) accm[a] = 0.0f;
        if (inside) {
            const float dv = vp.data[o * rec + (int64_t)Y * prm.out_nx + X];
            const float cT = dv * ib2, cO = O * ib2;
#pragma unroll
            for (int a = 0; a < 6; ++a) {
                acc[a] = cT * J[a];
                acc[6 + a] = cO * J[a];
            }
            if (leader) {
                acc[12] = O * O;
                acc[13] = O * dv;
                acc[14] = dv * dv;
#pragma unroll
                for (int i = 0; i < 6; ++i)
#pragma unroll
                    for (int j = i; j < 6; ++j) accm[pk(i, j)] = JB[i] * JB[j];
            }
        }
        warp_reduce_scatter<16>(acc, lane);
        warp_reduce_scatter<32>(accm, lane);
        float* rw = red + ((o - o_begin) * tile_y + wid) * kGnK;  // this warp's slot
        if (lane % 2 == 0 && lane / 2 < 15) rw[lane / 2] = acc[0];
        if (lane < 21) rw[15 + lane] = accm[0];
    }
    __syncthreads();
    const int no = (int)min((int64_t)opc, prm.n - o_begin);
    for (int i = tid; i < no * kGnK; i += blockDim.x) {
        const int ol = i / kGnK, k = i - ol * kGnK;
        float s2 = 0.0f;
        for (int wy = 0; wy < tile_y; ++wy) s2 += red[(ol * tile_y + wy) * kGnK + k];
        vp.partial[((o_begin + ol) * ntiles + t) * kGnK + k] = s2;
    }
}

// Gauss-Newton for records binned 2x2 or 4x4: CTAs of four warps over 32 x 4
// PPT pixel tiles, PPT pixel rows (layers of 32 x 4) per thread.  Per layer
// the warp sums each binning block's value and Jacobian by shuffles (as
// k_gn), and the block's first lane stores the block's eight numbers (J_B,
// O_B, T_B) in shared memory; after the last layer every lane forms one or
// two of the 36 products (21 of J J^T, J T, J O and the three dot products),
// summed over the warp's blocks of all layers.  The products are paid once
// per block instead of in every lane, and no warp reduction of the 36 sums
// is needed.
#ifndef EBSD_GN1_MIN_BLOCKS
#define EBSD_GN1_MIN_BLOCKS 5
#endif
template <int NV, int PPT>
__global__ void __launch_bounds__(128, EBSD_GN1_MIN_BLOCKS)
    k_gn1(const FwdParams prm, const VjpParams vp, int tiles_x, int ntiles, int opc)
{
    extern __shared__ float sm[];  // [opc][4 warps][36] warp sums, then per warp the blocks
    const int b = vp.binning;      // 2 or 4
    const int bpw = 32 / (b * b);  // binning blocks per warp and layer
    float* red = sm;
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    float* blk = sm + (size_t)opc * 4 * kGnK + (size_t)wid * PPT * 8 * 8;  // [PPT * bpw][8]
    int tx, ty;
    adj_pixel<true>(tid, b, tx, ty);
    const int bw = 32 / b;         // warp width in pixels
    const bool leader = (lane % bw) % b == 0 && (lane / bw) % b == 0;
    const int bidx = (lane % bw) / b;  // block of this lane within the warp's layer
    // the products this lane forms: operands (0..5 J_B, 6 O_B, 7 T_B) of
    // product j = lane and j = lane + 32, in the order of the partial sums
    auto operands = [](int j, int& u, int& v) {
        if (j < 6) {
            u = 7; v = j;
        } else if (j < 12) {
            u = 6; v = j - 6;
        } else if (j < 15) {
            u = j == 14 ? 7 : 6; v = j == 12 ? 6 : 7;
        } else {
            int k = j - 15, i = 0;
            while (k >= 6 - i) { k -= 6 - i; ++i; }
            u = i; v = i + k;
        }
    };
    int u0, v0, u1 = 0, v1 = 0;
    operands(lane, u0, v0);
    const bool two = lane + 32 < kGnK;
    if (two) operands(lane + 32, u1, v1);

    const unsigned n_ob = (unsigned)((prm.n + opc - 1) / opc);
    const int t = (int)(blockIdx.x / n_ob);
    const int64_t o_begin = (int64_t)(blockIdx.x % n_ob) * opc;
    const int x = (t % tiles_x) * kTileX + tx;
    const int y0 = (t / tiles_x) * (4 * PPT) + ty;
    const uint64_t pol = l2_policy_evict_last();
    const float pref = (float)prm.prefactor;
    const float ib2 = 1.0f / (float)(b * b);
    const int64_t rec = (int64_t)prm.out_nx * prm.out_ny;
    const int nblk = PPT * bpw;

    for (int64_t o = o_begin; o < o_begin + opc && o < prm.n; ++o) {
#pragma unroll 1
        for (int k = 0; k < PPT; ++k) {
            const int y = y0 + 4 * k;
            // only pixels of full output blocks contribute (binning crops to the floor)
            const bool inside = x < prm.numsx && y < prm.numsy && x < prm.out_nx * b &&
                                y < prm.out_ny * b;
            float val = 0.0f, J[6] = {0, 0, 0, 0, 0, 0};
            if (inside) pixel_value_jacobian<NV>(prm, vp, y * prm.numsx + x, o, pol, pref, val, J);
            const float O = adj_block_sum(val, b) * ib2;
            float JB[6];
#pragma unroll
            for (int a = 0; a < 6; ++a) JB[a] = adj_block_sum(J[a], b) * ib2;
            if (leader) {
                // a block lies wholly inside or wholly outside (then all zeros)
                const float dv =
                    inside ? vp.data[o * rec + (int64_t)(y / b) * prm.out_nx + x / b] : 0.0f;
                float4* e = reinterpret_cast<float4*>(blk + (k * bpw + bidx) * 8);
                e[0] = make_float4(JB[0], JB[1], JB[2], JB[3]);
                e[1] = make_float4(JB[4], JB[5], O, dv);
            }
        }
        __syncwarp();
        float s0 = 0.0f, s1 = 0.0f;
        for (int i = 0; i < nblk; ++i) {
            const float* e = blk + i * 8;
            s0 = fmaf(e[u0], e[v0], s0);
            if (two) s1 = fmaf(e[u1], e[v1], s1);
        }
        float* rw = red + ((o - o_begin) * 4 + wid) * kGnK;
        rw[lane] = s0;
        if (two) rw[lane + 32] = s1;
        __syncwarp();  // the blocks of the next orientation overwrite these
    }
    __syncthreads();
    const int no = (int)min((int64_t)opc, prm.n - o_begin);
    for (int i = tid; i < no * kGnK; i += blockDim.x) {
        const int ol = i / kGnK, k = i - ol * kGnK;
        float s2 = 0.0f;
        for (int w = 0; w < 4; ++w) s2 += red[(ol * 4 + w) * kGnK + k];
        vp.partial[((o_begin + ol) * ntiles + t) * kGnK + k] = s2;
    }
}

// Per orientation: binary64 sums of the partials, then H, g and the loss.
__global__ void k_gn_reduce(const float* __restrict__ partial, int64_t n, int ntiles,
                            double* __restrict__ sys, float* __restrict__ loss)
{
    const int64_t o = (int64_t)blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (o >= n) return;
    double sacc[kGnK];
#pragma unroll
    for (int a = 0; a < kGnK; ++a) sacc[a] = 0.0;
    for (int t = lane; t < ntiles; t += 32) {
        const float* pp = partial + ((int64_t)o * ntiles + t) * kGnK;
#pragma unroll
        for (int a = 0; a < kGnK; ++a) sacc[a] += (double)pp[a];
    }
#pragma unroll
    for (int a = 0; a < kGnK; ++a)
        for (int off = 16; off > 0; off >>= 1) sacc[a] += __shfl_xor_sync(0xffffffffu, sacc[a], off);
    if (lane != 0) return;
    double* out = sys + o * kGnSys;
    const double soo = sacc[12], sot = sacc[13], stt = sacc[14];
    if (!(soo > 0.0) || !(stt > 0.0)) {
        for (int a = 0; a < kGnSys; ++a) out[a] = 0.0;
        if (loss) loss[o] = 0.0f;
        return;
    }
    const double nO = sqrt(soo), nT = sqrt(stt), cosv = sot / (nO * nT);
    double av[6];
    for (int i = 0; i < 6; ++i) av[i] = sacc[6 + i] / nO;
    for (int i = 0; i < 6; ++i)
        for (int j = i; j < 6; ++j)
            out[pk(i, j)] = (sacc[15 + pk(i, j)] - av[i] * av[j]) / soo;
    for (int i = 0; i < 6; ++i) out[21 + i] = (av[i] * cosv - sacc[i] / nT) / nO;
    out[27] = 1.0 - cosv;
    if (loss) loss[o] = (float)(1.0 - cosv);
}

__device__ __forceinline__ double hget(const double* sys, int i, int j)
{
    return i <= j ? sys[pk(i, j)] : sys[pk(j, i)];
}

// inverse of a symmetric 3x3 (row-major); false if not positive definite
__device__ __forceinline__ bool inv3(const double A[9], double Ai[9])
{
    const double c00 = A[4] * A[8] - A[5] * A[7], c01 = A[5] * A[6] - A[3] * A[8],
                 c02 = A[3] * A[7] - A[4] * A[6];
    const double det = A[0] * c00 + A[1] * c01 + A[2] * c02;
    if (!(det > 0.0) || !isfinite(det)) return false;
    const double id = 1.0 / det;
    Ai[0] = c00 * id;
    Ai[1] = (A[2] * A[7] - A[1] * A[8]) * id;
    Ai[2] = (A[1] * A[5] - A[2] * A[4]) * id;
    Ai[3] = c01 * id;
    Ai[4] = (A[0] * A[8] - A[2] * A[6]) * id;
    Ai[5] = (A[2] * A[3] - A[0] * A[5]) * id;
    Ai[6] = c02 * id;
    Ai[7] = (A[1] * A[6] - A[0] * A[7]) * id;
    Ai[8] = (A[0] * A[4] - A[1] * A[3]) * id;
    return true;
}

// damped rotation block A = H_rr + lambda diag(H_rr)
__device__ __forceinline__ void rot_block(const double* sys, double lambda, double A[9])
{
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) A[i * 3 + j] = hget(sys, i, j);
    for (int i = 0; i < 3; ++i) A[i * 4] *= 1.0 + lambda;
}

// Pattern-centre Schur complement: sum over patterns of
//   S_n = C_n - B_n^T A_n^-1 B_n,  r_n = -(g_p - B_n^T A_n^-1 g_r),
// in binary64, one partial per block (fixed order), 12 numbers each.
__global__ void k_gn_schur(const double* __restrict__ sys, int64_t n, double lambda,
                           double* __restrict__ partial)
{
    __shared__ double sh[256][12];
    const int64_t o = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    double v[12];
    for (int a = 0; a < 12; ++a) v[a] = 0.0;
    if (o < n) {
        const double* sp = sys + o * kGnSys;
        double A[9], Ai[9];
        rot_block(sp, lambda, A);
        if (inv3(A, Ai)) {
            double B[3][3], AiB[3][3], Aig[3];
            for (int i = 0; i < 3; ++i)
                for (int j = 0; j < 3; ++j) B[i][j] = hget(sp, i, 3 + j);
            for (int i = 0; i < 3; ++i) {
                Aig[i] = 0.0;
                for (int k = 0; k < 3; ++k) Aig[i] += Ai[i * 3 + k] * sp[21 + k];
                for (int j = 0; j < 3; ++j) {
                    AiB[i][j] = 0.0;
                    for (int k = 0; k < 3; ++k) AiB[i][j] += Ai[i * 3 + k] * B[k][j];
                }
            }
            for (int i = 0; i < 3; ++i) {
                for (int j = 0; j < 3; ++j) {
                    double bab = 0.0;
                    for (int k = 0; k < 3; ++k) bab += B[k][i] * AiB[k][j];
                    v[i * 3 + j] = hget(sp, 3 + i, 3 + j) - bab;
                }
                double bag = 0.0;
                for (int k = 0; k < 3; ++k) bag += B[k][i] * Aig[k];
                v[9 + i] = -(sp[24 + i] - bag);
            }
        }
    }
    for (int a = 0; a < 12; ++a) sh[threadIdx.x][a] = v[a];
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w)
            for (int a = 0; a < 12; ++a) sh[threadIdx.x][a] += sh[threadIdx.x + w][a];
        __syncthreads();
    }
    if (threadIdx.x < 12) partial[(int64_t)blockIdx.x * 12 + threadIdx.x] = sh[0][threadIdx.x];
}

__global__ void k_gn_schur_final(const double* __restrict__ partial, int nblocks,
                                 double* __restrict__ out)
{
    if (threadIdx.x >= 12) return;
    double s2 = 0.0;
    for (int bk = 0; bk < nblocks; ++bk) s2 += partial[(int64_t)bk * 12 + threadIdx.x];
    out[threadIdx.x] = s2;
}

// Per pattern: d_rot = -A^-1 (g_r + B dpc), q <- exp(d_rot) (x) q, renormalised.
__global__ void k_gn_update(const double* __restrict__ sys, int64_t n, double lambda,
                            const double* __restrict__ dpc, float4* __restrict__ quats,
                            float* __restrict__ step)
{
    const int64_t o = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= n) return;
    const double* sp = sys + o * kGnSys;
    double A[9], Ai[9], rhs[3];
    rot_block(sp, lambda, A);
    for (int i = 0; i < 3; ++i) {
        rhs[i] = sp[21 + i];
        if (dpc)
            for (int j = 0; j < 3; ++j) rhs[i] += hget(sp, i, 3 + j) * dpc[j];
    }
    double w[3] = {0.0, 0.0, 0.0};
    if (inv3(A, Ai))
        for (int i = 0; i < 3; ++i)
            w[i] = -(Ai[i * 3] * rhs[0] + Ai[i * 3 + 1] * rhs[1] + Ai[i * 3 + 2] * rhs[2]);
    const double th = sqrt(w[0] * w[0] + w[1] * w[1] + w[2] * w[2]);
    step[o] = (float)th;
    if (!(th > 0.0) || !isfinite(th)) return;
    const double c = cos(0.5 * th), sn = sin(0.5 * th) / th;
    const double e0 = c, e1 = sn * w[0], e2 = sn * w[1], e3 = sn * w[2];
    const float4 q = quats[o];
    double r0 = e0 * q.x - e1 * q.y - e2 * q.z - e3 * q.w;
    double r1 = e0 * q.y + e1 * q.x + e2 * q.w - e3 * q.z;
    double r2 = e0 * q.z - e1 * q.w + e2 * q.x + e3 * q.y;
    double r3 = e0 * q.w + e1 * q.z - e2 * q.y + e3 * q.x;
    const double nq = sqrt(r0 * r0 + r1 * r1 + r2 * r2 + r3 * r3);
    quats[o] = make_float4((float)(r0 / nq), (float)(r1 / nq), (float)(r2 / nq), (float)(r3 / nq));
}

// Dynamic shared memory above the default 48 KB needs the kernel's opt-in.
template <typename Kern>
cudaError_t allow_smem(Kern kern, size_t bytes)
{
    if (bytes <= 48 * 1024) return cudaSuccess;
    return cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

template <int NV>
cudaError_t launch_gn_nv(const FwdParams& p, const VjpParams& vp, int tile_y, cudaStream_t s)
{
    if ((vp.binning == 2 || vp.binning == 4) && tile_y % 4 == 0 && tile_y <= 32) {
        // binned 2x2 / 4x4: four warps, tile_y / 4 pixel rows per thread
        const int tiles_x = (p.numsx + kTileX - 1) / kTileX;
        const int ntiles = tiles_x * ((p.numsy + tile_y - 1) / tile_y);
        const int opc = vp.opc;
        const int64_t blocks = ((p.n + opc - 1) / opc) * ntiles;
        if (blocks > 0x7fffffffLL) return cudaErrorInvalidConfiguration;
        const int ppt = tile_y / 4;
        const size_t smem = sizeof(float) * ((size_t)opc * 4 * kGnK + (size_t)4 * ppt * 64);
        auto go = [&](auto kern) {
            const cudaError_t e = allow_smem(kern, smem);
            if (e != cudaSuccess) return e;
            kern<<<(unsigned)blocks, 128, smem, s>>>(p, vp, tiles_x, ntiles, opc);
            return cudaGetLastError();
        };
        return ppt == 1   ? go(k_gn1<NV, 1>)
               : ppt == 2 ? go(k_gn1<NV, 2>)
               : ppt == 4 ? go(k_gn1<NV, 4>)
                          : go(k_gn1<NV, 8>);
    }
    const int tiles_x = (p.numsx + kTileX - 1) / kTileX;
    const int tiles_y = (p.numsy + tile_y - 1) / tile_y;
    const int ntiles = tiles_x * tiles_y;
    const int opc = vp.opc;
    const int64_t blocks = ((p.n + opc - 1) / opc) * ntiles;
    if (blocks > 0x7fffffffLL) return cudaErrorInvalidConfiguration;
    const size_t smem = sizeof(float) * (33 * tile_y * 7 + (size_t)kGnK * tile_y * opc);
    const bool bsh = vp.binning == 2 || vp.binning == 4;
    auto go = [&](auto kern) {
        const cudaError_t e = allow_smem(kern, smem);
        if (e != cudaSuccess) return e;
        kern<<<(unsigned)blocks, kTileX * tile_y, smem, s>>>(p, vp, tile_y, tiles_x, ntiles, opc);
        return cudaGetLastError();
    };
    return bsh ? go(k_gn<NV, true>) : go(k_gn<NV, false>);
}

template <int NV>
cudaError_t launch_vjp_nv(const FwdParams& p, const VjpParams& vp, int mode, int tile_y,
                          cudaStream_t s)
{
    const int tiles_x = (p.numsx + kTileX - 1) / kTileX;
    const int tiles_y = (p.numsy + tile_y - 1) / tile_y;
    const int ntiles = tiles_x * tiles_y;
    const int opc = vp.opc;
    const int64_t blocks = ((p.n + opc - 1) / opc) * ntiles;
    if (blocks > 0x7fffffffLL) return cudaErrorInvalidConfiguration;
    const int K = mode == EBSD_VJP_NDP ? 15 : 6;
    if (vp.binning == 1 && tile_y % 4 == 0 && tile_y <= 32) {
        // unbinned: four warps, tile_y / 4 pixels per thread
        const size_t smem1 = sizeof(float) * (size_t)K * 4 * opc;
        auto go1 = [&](auto kern) {
            const cudaError_t e = allow_smem(kern, smem1);
            if (e != cudaSuccess) return e;
            kern<<<(unsigned)blocks, 128, smem1, s>>>(p, vp, tiles_x, ntiles, opc);
            return cudaGetLastError();
        };
        const int ppt = tile_y / 4;
        if (mode == EBSD_VJP_NDP)
            return ppt == 1   ? go1(k_vjp1<NV, EBSD_VJP_NDP, 1>)
                   : ppt == 2 ? go1(k_vjp1<NV, EBSD_VJP_NDP, 2>)
                   : ppt == 4 ? go1(k_vjp1<NV, EBSD_VJP_NDP, 4>)
                              : go1(k_vjp1<NV, EBSD_VJP_NDP, 8>);
        return ppt == 1   ? go1(k_vjp1<NV, EBSD_VJP_COTANGENT, 1>)
               : ppt == 2 ? go1(k_vjp1<NV, EBSD_VJP_COTANGENT, 2>)
               : ppt == 4 ? go1(k_vjp1<NV, EBSD_VJP_COTANGENT, 4>)
                          : go1(k_vjp1<NV, EBSD_VJP_COTANGENT, 8>);
    }
    const size_t smem = sizeof(float) * (33 * tile_y + (size_t)K * tile_y * opc);
    const bool bsh = vp.binning == 2 || vp.binning == 4;
    auto go = [&](auto kern) {
        const cudaError_t e = allow_smem(kern, smem);
        if (e != cudaSuccess) return e;
        kern<<<(unsigned)blocks, kTileX * tile_y, smem, s>>>(p, vp, tile_y, tiles_x, ntiles, opc);
        return cudaGetLastError();
    };
    if (mode == EBSD_VJP_NDP)
        return bsh ? go(k_vjp<NV, EBSD_VJP_NDP, true>) : go(k_vjp<NV, EBSD_VJP_NDP, false>);
    return bsh ? go(k_vjp<NV, EBSD_VJP_COTANGENT, true>)
               : go(k_vjp<NV, EBSD_VJP_COTANGENT, false>);
}

}  // namespace

int vjp_tiles(const FwdParams& p, int tile_y)
{
    return ((p.numsx + kTileX - 1) / kTileX) * ((p.numsy + tile_y - 1) / tile_y);
}

cudaError_t launch_vjp(const FwdParams& p, const VjpParams& vp, int NV, int mode, int tile_y,
                       cudaStream_t s)
{
    if (p.n <= 0) return cudaSuccess;
    cudaError_t e;
    switch (NV) {
        case 1: e = launch_vjp_nv<1>(p, vp, mode, tile_y, s); break;
        case 2: e = launch_vjp_nv<2>(p, vp, mode, tile_y, s); break;
        case 3: e = launch_vjp_nv<3>(p, vp, mode, tile_y, s); break;
        case 4: e = launch_vjp_nv<4>(p, vp, mode, tile_y, s); break;
        case 5: e = launch_vjp_nv<5>(p, vp, mode, tile_y, s); break;
        case 6: e = launch_vjp_nv<6>(p, vp, mode, tile_y, s); break;
        case 7: e = launch_vjp_nv<7>(p, vp, mode, tile_y, s); break;
        case 8: e = launch_vjp_nv<8>(p, vp, mode, tile_y, s); break;
        default: return cudaErrorInvalidValue;
    }
    if (e != cudaSuccess) return e;
    const int ntiles = vjp_tiles(p, tile_y);
    const int wpb = 8;
    const unsigned rb = (unsigned)((p.n + wpb - 1) / wpb);
    if (mode == EBSD_VJP_NDP)
        k_vjp_reduce<EBSD_VJP_NDP><<<rb, 32 * wpb, 0, s>>>(vp.partial, p.n, ntiles, vp.loss,
                                                           vp.grad);
    else
        k_vjp_reduce<EBSD_VJP_COTANGENT><<<rb, 32 * wpb, 0, s>>>(vp.partial, p.n, ntiles, vp.loss,
                                                                 vp.grad);
    return cudaGetLastError();
}

cudaError_t launch_gn_accumulate(const FwdParams& p, const VjpParams& vp, int NV, int tile_y,
                                 double* sys, float* loss, cudaStream_t s)
{
    if (p.n <= 0) return cudaSuccess;
    cudaError_t e;
    switch (NV) {
        case 1: e = launch_gn_nv<1>(p, vp, tile_y, s); break;
        case 2: e = launch_gn_nv<2>(p, vp, tile_y, s); break;
        case 3: e = launch_gn_nv<3>(p, vp, tile_y, s); break;
        case 4: e = launch_gn_nv<4>(p, vp, tile_y, s); break;
        case 5: e = launch_gn_nv<5>(p, vp, tile_y, s); break;
        case 6: e = launch_gn_nv<6>(p, vp, tile_y, s); break;
        case 7: e = launch_gn_nv<7>(p, vp, tile_y, s); break;
        case 8: e = launch_gn_nv<8>(p, vp, tile_y, s); break;
        default: return cudaErrorInvalidValue;
    }
    if (e != cudaSuccess) return e;
    const int ntiles = vjp_tiles(p, tile_y);
    const int wpb = 4;
    k_gn_reduce<<<(unsigned)((p.n + wpb - 1) / wpb), 32 * wpb, 0, s>>>(vp.partial, p.n, ntiles,
                                                                      sys, loss);
    return cudaGetLastError();
}

int gn_schur_blocks(int64_t n) { return (int)((n + 255) / 256); }

cudaError_t launch_gn_schur(const double* sys, int64_t n, double lambda, double* partial,
                            double* out, cudaStream_t s)
{
    const int nb = gn_schur_blocks(n);
    if (nb > 0) k_gn_schur<<<nb, 256, 0, s>>>(sys, n, lambda, partial);
    k_gn_schur_final<<<1, 32, 0, s>>>(partial, nb, out);
    return cudaGetLastError();
}

cudaError_t launch_gn_update(const double* sys, int64_t n, double lambda, const double* dpc,
                             float4* quats, float* step, cudaStream_t s)
{
    if (n <= 0) return cudaSuccess;
    k_gn_update<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(sys, n, lambda, dpc, quats, step);
    return cudaGetLastError();
}

}  // namespace ebsd
