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

template <int NV, int MODE>
__global__ void __launch_bounds__(256, 3) k_vjp(const FwdParams prm, const VjpParams vp,
                                                 int tile_y, int tiles_x, int ntiles, int opc)
{
    constexpr int K = MODE == EBSD_VJP_NDP ? 15 : 6;
    constexpr int KP = MODE == EBSD_VJP_NDP ? 16 : 8;
    extern __shared__ float sm[];  // [tile_y][33] pattern tile, then [tile_y][K] warp sums
    float* tile = sm;
    float* red = sm + 33 * tile_y;
    const int tid = threadIdx.x, tx = tid & 31, ty = tid >> 5;
    const int t = (int)(blockIdx.x % (unsigned)ntiles);
    const int64_t o_begin = (int64_t)(blockIdx.x / (unsigned)ntiles) * opc;
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
    const float pref = (float)prm.prefactor;
    const float ib2 = 1.0f / (float)(b * b);
    const int64_t rec = (int64_t)prm.out_nx * prm.out_ny;
    const int X = x / b, Y = y / b;
    const bool leader = (x % b == 0) && (y % b == 0);

    for (int64_t o = o_begin; o < o_begin + opc && o < prm.n; ++o) {
        float val = 0.0f, J[6] = {0, 0, 0, 0, 0, 0};
        if (inside) {
            const float4 q = __ldg(prm.quats + o);
            const float4 r = __ldg(prm.rg + p);
            float d0, d1, d2;
            rotate_direction(q, r.x, r.y, r.z, d0, d1, d2);
            const float nd = sqrtf(fmaf(d0, d0, fmaf(d1, d1, d2 * d2)));
            const float h0 = d0 / nd, h1 = d1 / nd, h2 = d2 / nd;
            float c0 = d0, c1 = d1, c2 = d2;
            normalize_fold(c0, c1, c2);
            const float s = h2 < 0.0f ? -1.0f : 1.0f;
            float LX, LY, dX[3], dY[3];
            lambert_inverse_jac(c0, c1, c2, prm.spi2, prm.accurate != 0, LX, LY, dX, dY);
            float dx, dy;
            int nix, niy;
            const int ix0 = lambert_cell(prm.scl * LX, prm.npx, dx, nix);
            const int iy0 = lambert_cell(prm.scl * LY, prm.npy, dy, niy);
            const int ix1 = min(ix0 + 1, 2 * prm.npx), iy1 = min(iy0 + 1, 2 * prm.npy);
            const float dxm = 1.0f - dx, dym = 1.0f - dy;
            const float4* m00 = prm.master + ((int64_t)iy0 * prm.gx + ix0) * NV;
            const float4* m10 = prm.master + ((int64_t)iy0 * prm.gx + ix1) * NV;
            const float4* m01 = prm.master + ((int64_t)iy1 * prm.gx + ix0) * NV;
            const float4* m11 = prm.master + ((int64_t)iy1 * prm.gx + ix1) * NV;
            float P = 0.0f, gX = 0.0f, gY = 0.0f, gW0 = 0.0f, gW1 = 0.0f, gW2 = 0.0f;
            // one float4 group of bins at a time: unrolling would hoist all
            // 7*NV vector loads and spill
#pragma unroll 1
            for (int c = 0; c < NV; ++c) {
                const float4 A = __ldg(m00 + c), B = __ldg(m10 + c), C = __ldg(m01 + c),
                             D = __ldg(m11 + c);
                const float4 wc = __ldg(prm.W + (int64_t)c * prm.P + p);
                const float4 e0 = __ldg(vp.dW + (int64_t)(0 * NV + c) * prm.P + p);
                const float4 e1 = __ldg(vp.dW + (int64_t)(1 * NV + c) * prm.P + p);
                const float4 e2 = __ldg(vp.dW + (int64_t)(2 * NV + c) * prm.P + p);
#define EBSD_BIN(f)                                                                        \
    {                                                                                      \
        const float bv = fmaf(A.f, dxm * dym, fmaf(B.f, dx * dym, fmaf(C.f, dxm * dy, D.f * dx * dy))); \
        P = fmaf(wc.f, bv, P);                                                              \
        gX = fmaf(wc.f, fmaf(B.f - A.f, dym, (D.f - C.f) * dy), gX);                         \
        gY = fmaf(wc.f, fmaf(C.f - A.f, dxm, (D.f - B.f) * dx), gY);                         \
        gW0 = fmaf(e0.f, bv, gW0);                                                          \
        gW1 = fmaf(e1.f, bv, gW1);                                                          \
        gW2 = fmaf(e2.f, bv, gW2);                                                          \
    }
                EBSD_BIN(x) EBSD_BIN(y) EBSD_BIN(z) EBSD_BIN(w)
#undef EBSD_BIN
            }
            val = pref * P;
            const float sx = prm.scl * pref * gX, sy = prm.scl * pref * gY;
            const float gc0 = sx * dX[0] + sy * dY[0];
            const float gc1 = sx * dX[1] + sy * dY[1];
            const float gc2 = sx * dX[2] + sy * dY[2];
            const float pr = gc0 * h0 + gc1 * h1 + gc2 * h2;
            const float k = s / nd;
            const float g0 = k * (gc0 - pr * h0), g1 = k * (gc1 - pr * h1), g2 = k * (gc2 - pr * h2);
            J[0] = d1 * g2 - d2 * g1;
            J[1] = d2 * g0 - d0 * g2;
            J[2] = d0 * g1 - d1 * g0;
            // M^T g = conj(q) (x) (0,g) (x) q
            const float u0 = -(g0 * q.y) - g1 * q.z - g2 * q.w;
            const float u1 = g0 * q.x + g1 * q.w - g2 * q.z;
            const float u2 = -(g0 * q.w) + g1 * q.x + g2 * q.y;
            const float u3 = g0 * q.z - g1 * q.y + g2 * q.x;
            const float m0 = q.x * u1 - q.y * u0 - q.z * u3 + q.w * u2;
            const float m1 = q.x * u2 + q.y * u3 - q.z * u0 - q.w * u1;
            const float m2 = q.x * u3 - q.y * u2 + q.z * u1 - q.w * u0;
            const float4 r0 = __ldg(vp.drg + p), r1 = __ldg(vp.drg + prm.P + p),
                         r2 = __ldg(vp.drg + 2 * (int64_t)prm.P + p);
            J[3] = m0 * r0.x + m1 * r0.y + m2 * r0.z + pref * gW0;
            J[4] = m0 * r1.x + m1 * r1.y + m2 * r1.z + pref * gW1;
            J[5] = m0 * r2.x + m1 * r2.y + m2 * r2.z + pref * gW2;
        }
        // output-record value of this pixel's block
        float O = val;
        if (b > 1) {
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
        warp_reduce_scatter<KP>(acc, tx);
        {
            const int idx = tx / (32 / KP);
            if (tx % (32 / KP) == 0 && idx < K) red[ty * K + idx] = acc[0];
        }
        __syncthreads();
        if (tid < K) {
            float s2 = 0.0f;
            for (int wy = 0; wy < tile_y; ++wy) s2 += red[wy * K + tid];
            vp.partial[(o * ntiles + t) * K + tid] = s2;
        }
        __syncthreads();
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
    const size_t smem = sizeof(float) * (33 * tile_y + K * tile_y);
    if (mode == EBSD_VJP_NDP)
        k_vjp<NV, EBSD_VJP_NDP><<<(unsigned)blocks, kTileX * tile_y, smem, s>>>(p, vp, tile_y,
                                                                               tiles_x, ntiles, opc);
    else
        k_vjp<NV, EBSD_VJP_COTANGENT><<<(unsigned)blocks, kTileX * tile_y, smem, s>>>(
            p, vp, tile_y, tiles_x, ntiles, opc);
    return cudaGetLastError();
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

}  // namespace ebsd
