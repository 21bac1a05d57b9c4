// Per-detector and per-master set-up kernels: master re-layout, detector
// direction cosines, Monte-Carlo energy weights and the num_el sum.
// Compiled with -fmad=false (see ebsd_device.cuh).
#include "ebsd_device.cuh"
#include "ebsd_internal.h"

namespace ebsd {

// sr = sum(srtmp,4) (CTEMEBSD.f90:404) restricted to bins e0..e0+nsel-1 and
// re-laid out energy-fastest: il[(y*pitch + x)*NV*4 + k], zero padded to
// NV*4 bins and to `pitch` nodes per row (master_pitch).  The Fortran source
// is srtmp(x, y, E, set), x fastest.
__global__ void k_master_relayout(const float* __restrict__ raw, int gx, int gy, int pitch,
                                  int nE, int numset, int e0, int nsel, int NV,
                                  float* __restrict__ il)
{
    const int64_t slot = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (slot >= (int64_t)pitch * gy) return;
    const int y = (int)(slot / pitch), x = (int)(slot - (int64_t)y * pitch);
    const int64_t plane = (int64_t)gx * gy;    // elements per energy bin
    const int64_t setstride = plane * nE;      // elements per atom set
    const int64_t node = (int64_t)y * gx + x;
    float* dst = il + slot * (int64_t)NV * 4;
    for (int k = 0; k < NV * 4; ++k) {
        float s = 0.0f;
        if (k < nsel && x < gx) {
            const float* src = raw + (int64_t)(e0 + k) * plane + node;
            for (int st = 0; st < numset; ++st) s = s + src[st * setstride];
        }
        dst[k] = s;
    }
}

cudaError_t launch_master_relayout(const float* raw, int npx, int npy, int nE, int numset,
                                   int e0, int nsel, int NV, float4* il, cudaStream_t s)
{
    const int gx = 2 * npx + 1, gy = 2 * npy + 1, pitch = master_pitch(npx, NV);
    const int64_t slots = (int64_t)pitch * gy;
    const int bs = 256;
    const unsigned blocks = (unsigned)((slots + bs - 1) / bs);
    k_master_relayout<<<blocks, bs, 0, s>>>(raw, gx, gy, pitch, nE, numset, e0, nsel, NV,
                                             reinterpret_cast<float*>(il));
    return cudaGetLastError();
}

// Detector direction cosines, CTEMEBSD.f90:416-452.  ca/sa are cos/sin of
// alp (:422-424) computed on the host as the reference does.  Pixel p =
// i + numsx*j (Fortran rgx(i,j)).
__global__ void k_detector(float L, float delta, int numsx, int numsy, float xpc, float ypc,
                           float ca, float sa, float4* __restrict__ rg)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y;
    if (i >= numsx || j >= numsy) return;
    const float scin_x = -((xpc - (1.0f - (float)numsx) * 0.5f - (float)i) * delta);  // :418
    const float scin_y = (ypc - (1.0f - (float)numsy) * 0.5f - (float)j) * delta;     // :419
    const float L2 = L * L;
    const float sx = L2 + scin_y * scin_y;                                              // :435
    const float Ls = ca * scin_y + L * sa;
    const float Lc = -(sa * scin_y) + L * ca;
    const float rhos = 1.0f / sqrtf(sx + scin_x * scin_x);                              // :439
    float x = Ls * rhos, y = scin_x * rhos, z = Lc * rhos;
    float n = x * x;                                                                     // :448
    n = n + y * y;
    n = n + z * z;
    n = sqrtf(n);
    rg[(int64_t)j * numsx + i] = make_float4(x / n, y / n, z / n, 0.0f);
}

cudaError_t launch_detector(const ebsd_geometry& g, float ca, float sa, float4* rg,
                            cudaStream_t s)
{
    dim3 grid((g.numsx + 127) / 128, g.numsy);
    k_detector<<<grid, 128, 0, s>>>(g.L, g.delta, g.numsx, g.numsy, g.xpc, g.ypc, ca, sa, rg);
    return cudaGetLastError();
}

// accum_e_detector for bins e0..e0+nsel-1, CTEMEBSD.f90:483-510 (the 0.25
// factor of :510 included).  accum_e(k, -nsx:nsx, -nsy:nsy), k fastest.
//
// Two evaluations per pixel:
//  * Wref: the reference's single-precision arithmetic on the single-precision
//    direction cosines rg; it only feeds num_el (:516), so the intensity
//    prefactor is the reference's;
//  * W: the weights the pattern kernels use.  With fp64 != 0 they are
//    evaluated in binary64 from the geometry (direction, Lambert map and
//    bilinear interpolation, as an FP64 re-evaluation of :416-510) and
//    rounded once; the sparse integer histogram makes the single-precision
//    weights carry ~1e-4 relative position noise, which binary64 removes.
//    With fp64 == 0, W = Wref.
// Both are stored as NV float4 planes of P pixels.
struct WeightsGeom {
    double L, delta, xpc, ypc, ca, sa;
    int numsx, numsy;
};

__device__ __forceinline__ void cell_f64(double ixy, int np, double& d, int& i0)
{
    const int ni = (int)((double)np + ixy) - np;
    d = ixy - (double)ni;
    i0 = ni + np;
    i0 = i0 < 0 ? 0 : (i0 > 2 * np ? 2 * np : i0);
}

__global__ void k_weights(const float4* __restrict__ rg, int P, const int32_t* __restrict__ acc,
                          int nE, int nsx, int nsy, float sclmc, float spi2, int e0, int nsel,
                          int NV, int fp64, WeightsGeom gd, float4* __restrict__ W,
                          float4* __restrict__ Wref)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= P) return;
    const int64_t gxm = 2 * nsx + 1;

    // --- reference single precision (feeds num_el) ---
    const float4 r = rg[p];
    float d0 = r.x, d1 = r.y, d2 = r.z;
    if (d2 < 0.0f) {                                                       // :488
        d0 = -d0;
        d1 = -d1;
        d2 = -d2;
    }
    float X, Y;
    lambert_inverse(d0, d1, d2, spi2, X, Y);                               // :490
    const float ixy0 = sclmc * Y;                                          // swap :491-493
    const float ixy1 = -(sclmc * X);
    float dx, dy;
    int nix, niy;
    const int ix0 = lambert_cell(ixy0, nsx, dx, nix);                      // :495-500
    const int iy0 = lambert_cell(ixy1, nsy, dy, niy);
    const float dxm = 1.0f - dx, dym = 1.0f - dy;
    const int ix1 = min(ix0 + 1, 2 * nsx), iy1 = min(iy0 + 1, 2 * nsy);
    const int32_t* a00 = acc + ((int64_t)iy0 * gxm + ix0) * nE + e0;
    const int32_t* a10 = acc + ((int64_t)iy0 * gxm + ix1) * nE + e0;
    const int32_t* a01 = acc + ((int64_t)iy1 * gxm + ix0) * nE + e0;
    const int32_t* a11 = acc + ((int64_t)iy1 * gxm + ix1) * nE + e0;

    // --- binary64 re-evaluation (feeds the pattern kernels) ---
    double Dx = 0.0, Dy = 0.0;
    int jx0 = 0, jy0 = 0, jx1 = 0, jy1 = 0;
    if (fp64) {
        const int i = p % gd.numsx, j = p / gd.numsx;
        const double sxp = -(gd.xpc - (1.0 - gd.numsx) * 0.5 - i) * gd.delta;
        const double syp = (gd.ypc - (1.0 - gd.numsy) * 0.5 - j) * gd.delta;
        const double Ls = gd.ca * syp + gd.L * gd.sa;
        const double Lc = -gd.sa * syp + gd.L * gd.ca;
        const double rh = 1.0 / sqrt(gd.L * gd.L + syp * syp + sxp * sxp);
        double x = Ls * rh, y = sxp * rh, z = Lc * rh;
        const double n = sqrt(x * x + y * y + z * z);
        x /= n;
        y /= n;
        z /= n;
        if (z < 0.0) {
            x = -x;
            y = -y;
            z = -z;
        }
        const double spi2d = 0.88622692545275801365;  // sqrt(pi)/2
        double LX = 0.0, LY = 0.0;
        const double s2 = x * x + y * y + z * z;
        if (!(fabs(1.0 - s2) > 1.0e-12) && fabs(z) != 1.0) {
            if (fabs(y) <= fabs(x)) {
                const double q = copysign(sqrt(2.0 * (1.0 - z)), x);
                LX = q * spi2d;
                LY = q * atan(y / x) / spi2d;
            } else {
                const double q = copysign(sqrt(2.0 * (1.0 - z)), y);
                LX = q * atan(x / y) / spi2d;
                LY = q * spi2d;
            }
        }
        const double scl = (double)nsx / 1.25331413731550025121;  // nsx / sqrt(pi/2)
        cell_f64(scl * LY, nsx, Dx, jx0);
        cell_f64(-(scl * LX), nsy, Dy, jy0);
        jx1 = min(jx0 + 1, 2 * nsx);
        jy1 = min(jy0 + 1, 2 * nsy);
    }
    const int32_t* b00 = acc + ((int64_t)jy0 * gxm + jx0) * nE + e0;
    const int32_t* b10 = acc + ((int64_t)jy0 * gxm + jx1) * nE + e0;
    const int32_t* b01 = acc + ((int64_t)jy1 * gxm + jx0) * nE + e0;
    const int32_t* b11 = acc + ((int64_t)jy1 * gxm + jx1) * nE + e0;
    const double Dxm = 1.0 - Dx, Dym = 1.0 - Dy;

    for (int c = 0; c < NV; ++c) {
        float v[4], u[4];
        for (int t = 0; t < 4; ++t) {
            const int k = 4 * c + t;
            float w = 0.0f, wd = 0.0f;
            if (k < nsel) {
                w = (float)a00[k] * dxm * dym + (float)a10[k] * dx * dym +      // :503-506
                    (float)a01[k] * dxm * dy + (float)a11[k] * dx * dy;
                w = w * 0.25f;                                                  // :510
                if (fp64)
                    wd = (float)(0.25 * ((double)b00[k] * Dxm * Dym + (double)b10[k] * Dx * Dym +
                                         (double)b01[k] * Dxm * Dy + (double)b11[k] * Dx * Dy));
                else
                    wd = w;
            }
            v[t] = w;
            u[t] = wd;
        }
        Wref[(int64_t)c * P + p] = make_float4(v[0], v[1], v[2], v[3]);
        W[(int64_t)c * P + p] = make_float4(u[0], u[1], u[2], u[3]);
    }
}

cudaError_t launch_weights(const float4* rg, int P, const int32_t* accum_e, int nE, int nsx,
                           int nsy, float sclmc, float spi2, int e0, int nsel, int NV, int fp64,
                           const ebsd_geometry& g, float4* W, float4* Wref, cudaStream_t s)
{
    WeightsGeom gd;
    const double dtor = (double)0.0174533f;
    const double alp = 0.5 * 3.141592653589793238 - ((double)(float)g.sig - (double)g.thetac) * dtor;
    gd.L = g.L;
    gd.delta = g.delta;
    gd.xpc = g.xpc;
    gd.ypc = g.ypc;
    gd.ca = cos(alp);
    gd.sa = sin(alp);
    gd.numsx = g.numsx;
    gd.numsy = g.numsy;
    const int bs = 256;
    k_weights<<<(P + bs - 1) / bs, bs, 0, s>>>(rg, P, accum_e, nE, nsx, nsy, sclmc, spi2, e0,
                                               nsel, NV, fp64, gd, W, Wref);
    return cudaGetLastError();
}

// Detector direction cosines in binary64 (the FP64 re-evaluation of
// CTEMEBSD.f90:416-452 that the binary64-geometry pattern kernel starts
// from): three planes x, y, z of P doubles, pixel p = i + numsx*j.
__global__ void k_detector64(WeightsGeom gd, double* __restrict__ rg64)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y;
    if (i >= gd.numsx || j >= gd.numsy) return;
    const double sxp = -(gd.xpc - (1.0 - gd.numsx) * 0.5 - i) * gd.delta;
    const double syp = (gd.ypc - (1.0 - gd.numsy) * 0.5 - j) * gd.delta;
    const double Ls = gd.ca * syp + gd.L * gd.sa;
    const double Lc = -gd.sa * syp + gd.L * gd.ca;
    const double rh = 1.0 / sqrt(gd.L * gd.L + syp * syp + sxp * sxp);
    const double x = Ls * rh, y = sxp * rh, z = Lc * rh;
    const double n = sqrt(x * x + y * y + z * z);
    const int64_t P = (int64_t)gd.numsx * gd.numsy, p = (int64_t)j * gd.numsx + i;
    rg64[p] = x / n;
    rg64[P + p] = y / n;
    rg64[2 * P + p] = z / n;
}

cudaError_t launch_detector64(const ebsd_geometry& g, double* rg64, cudaStream_t s)
{
    WeightsGeom gd;
    const double dtor = (double)0.0174533f;
    const double alp = 0.5 * 3.141592653589793238 - ((double)(float)g.sig - (double)g.thetac) * dtor;
    gd.L = g.L;
    gd.delta = g.delta;
    gd.xpc = g.xpc;
    gd.ypc = g.ypc;
    gd.ca = cos(alp);
    gd.sa = sin(alp);
    gd.numsx = g.numsx;
    gd.numsy = g.numsy;
    dim3 grid((g.numsx + 127) / 128, g.numsy);
    k_detector64<<<grid, 128, 0, s>>>(gd, rg64);
    return cudaGetLastError();
}

// num_el = nint(sum(accum_e_detector)), CTEMEBSD.f90:516.  gfortran sums
// the array sequentially in single precision in memory order (bin fastest,
// then x, then y); bins outside the window add exact zeros, and so do the
// zero-padded bins of the last float4 (s + 0 = s, s is never -0).  That order
// is one dependent chain of adds, which thread 0 runs out of shared memory
// while the whole CTA stages the next chunk of pixels (coalesced loads,
// double-buffered), so the chain runs at the add latency.  Runs once per
// detector.
template <int NV>
__global__ void __launch_bounds__(1024) k_num_el(const float4* __restrict__ W, int P,
                                                 float* __restrict__ out)
{
    constexpr int CH = 3072 / NV;            // pixels per chunk: 2 x 48 KB of float4
    extern __shared__ float4 stage[];        // [2][CH][NV]
    const int nch = (P + CH - 1) / CH;
    auto load = [&](int ch, int buf) {
        for (int i = threadIdx.x; i < CH * NV; i += blockDim.x) {
            const int c = i / CH, j = i - c * CH;  // plane by plane: coalesced
            const int p = ch * CH + j;
            stage[(buf * CH + j) * NV + c] =
                p < P ? W[(int64_t)c * P + p] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        }
    };
    float s = 0.0f;
    if (nch > 0) load(0, 0);
    __syncthreads();
    for (int ch = 0; ch < nch; ++ch) {
        if (ch + 1 < nch) load(ch + 1, (ch + 1) & 1);
        if (threadIdx.x == 0) {
            const float4* v = stage + (ch & 1) * CH * NV;
#pragma unroll 4
            for (int k = 0; k < CH * NV; ++k) {
                const float4 w = v[k];
                s = s + w.x;
                s = s + w.y;
                s = s + w.z;
                s = s + w.w;
            }
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = s;
}

cudaError_t launch_num_el(const float4* W, int P, int nsel, int NV, float* sum_out,
                          cudaStream_t s)
{
    (void)nsel;  // bins past nsel are zero in W
    switch (NV) {
#define EBSD_NUM_EL(n)                                                                    \
    case n: {                                                                             \
        const int bytes = (int)(sizeof(float4) * 2 * (3072 / n) * n);                    \
        const cudaError_t e = cudaFuncSetAttribute(                                       \
            k_num_el<n>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);             \
        if (e != cudaSuccess) return e;                                                   \
        k_num_el<n><<<1, 1024, bytes, s>>>(W, P, sum_out);                                \
        break;                                                                            \
    }
        EBSD_NUM_EL(1) EBSD_NUM_EL(2) EBSD_NUM_EL(3) EBSD_NUM_EL(4) EBSD_NUM_EL(5) EBSD_NUM_EL(6)
        EBSD_NUM_EL(7) EBSD_NUM_EL(8) EBSD_NUM_EL(9) EBSD_NUM_EL(10) EBSD_NUM_EL(11)
        EBSD_NUM_EL(12) EBSD_NUM_EL(13) EBSD_NUM_EL(14) EBSD_NUM_EL(15) EBSD_NUM_EL(16)
#undef EBSD_NUM_EL
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

}  // namespace ebsd

namespace ebsd {

// Derivatives of the detector quantities with respect to the pattern centre
// (xpc, ypc in pixels; L in microns), evaluated in binary64:
//   drg[a][p] = d rg(p) / d theta_a, rg = v/|v| with v the unnormalised
//               direction of CTEMEBSD.f90:434-442;
//   dW[a][c][p] = d W(p) / d theta_a for the window bins (float4 planes),
//               through the Lambert point of rg on the MC grid (:486-506).
// The cell indices are locally constant, so only the bilinear fractions
// carry derivatives.
__global__ void k_geom_derivs(WeightsGeom gd, const int32_t* __restrict__ acc, int nE, int nsx,
                              int nsy, int e0, int nsel, int NV, float4* __restrict__ drg,
                              float4* __restrict__ dW, int P)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= P) return;
    const int i = p % gd.numsx, j = p / gd.numsx;
    const double sxp = -(gd.xpc - (1.0 - gd.numsx) * 0.5 - i) * gd.delta;
    const double syp = (gd.ypc - (1.0 - gd.numsy) * 0.5 - j) * gd.delta;
    const double v[3] = {gd.ca * syp + gd.L * gd.sa, sxp, -gd.sa * syp + gd.L * gd.ca};
    const double nv = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    const double r[3] = {v[0] / nv, v[1] / nv, v[2] / nv};
    const double dv[3][3] = {{0.0, -gd.delta, 0.0},
                             {gd.ca * gd.delta, 0.0, -gd.sa * gd.delta},
                             {gd.sa, 0.0, gd.ca}};
    double dr[3][3];
    for (int a = 0; a < 3; ++a) {
        const double pr = r[0] * dv[a][0] + r[1] * dv[a][1] + r[2] * dv[a][2];
        for (int c = 0; c < 3; ++c) dr[a][c] = (dv[a][c] - pr * r[c]) / nv;
        drg[(int64_t)a * P + p] = make_float4((float)dr[a][0], (float)dr[a][1], (float)dr[a][2],
                                              0.0f);  // .w: d Dx / d theta_a, below
    }
    // MC Lambert point and its Jacobian (Lambert.f90:452-483 differentiated)
    double x = r[0], y = r[1], z = r[2], sm = 1.0;
    if (z < 0.0) {
        x = -x;
        y = -y;
        z = -z;
        sm = -1.0;
    }
    const double spi2 = 0.88622692545275801365;
    double LX = 0.0, LY = 0.0, dX[3] = {0, 0, 0}, dY[3] = {0, 0, 0};
    const double rxy = x * x + y * y;
    if (fabs(z) != 1.0 && rxy > 0.0) {
        const double rho = sqrt(2.0 * (1.0 - z));
        if (fabs(y) <= fabs(x)) {
            const double sg = copysign(1.0, x), a = atan(y / x);
            LX = sg * rho * spi2;
            LY = sg * rho * a / spi2;
            dX[2] = -sg * spi2 / rho;
            dY[0] = sg * rho / spi2 * (-y / rxy);
            dY[1] = sg * rho / spi2 * (x / rxy);
            dY[2] = -sg * a / (spi2 * rho);
        } else {
            const double sg = copysign(1.0, y), b = atan(x / y);
            LX = sg * rho * b / spi2;
            LY = sg * rho * spi2;
            dX[0] = sg * rho / spi2 * (y / rxy);
            dX[1] = sg * rho / spi2 * (-x / rxy);
            dX[2] = -sg * b / (spi2 * rho);
            dY[2] = -sg * spi2 / rho;
        }
    }
    const double scl = (double)nsx / 1.25331413731550025121;
    double Dx, Dy;
    int jx0, jy0;
    cell_f64(scl * LY, nsx, Dx, jx0);
    cell_f64(-(scl * LX), nsy, Dy, jy0);
    const int jx1 = min(jx0 + 1, 2 * nsx), jy1 = min(jy0 + 1, 2 * nsy);
    const double Dxm = 1.0 - Dx, Dym = 1.0 - Dy;
    double di0[3], di1[3];
    for (int a = 0; a < 3; ++a) {
        di0[a] = scl * sm * (dY[0] * dr[a][0] + dY[1] * dr[a][1] + dY[2] * dr[a][2]);
        di1[a] = -scl * sm * (dX[0] * dr[a][0] + dX[1] * dr[a][1] + dX[2] * dr[a][2]);
    }
    const int64_t gxm = 2 * nsx + 1;
    const int32_t* a00 = acc + ((int64_t)jy0 * gxm + jx0) * nE + e0;
    const int32_t* a10 = acc + ((int64_t)jy0 * gxm + jx1) * nE + e0;
    const int32_t* a01 = acc + ((int64_t)jy1 * gxm + jx0) * nE + e0;
    const int32_t* a11 = acc + ((int64_t)jy1 * gxm + jx1) * nE + e0;
    // dW_k / d theta_a = G0_k di0[a] + G1_k di1[a]: the slopes of the bilinear
    // weight along the two MC grid axes (planes 0..NV-1 and NV..2NV-1 of dW)
    // and the derivatives of the grid fractions (di0 in the drg planes' w,
    // di1 in plane 2NV of dW)
    for (int c = 0; c < NV; ++c) {
        float u0[4], u1[4];
        for (int t = 0; t < 4; ++t) {
            const int k = 4 * c + t;
            double g0 = 0.0, g1 = 0.0;
            if (k < nsel) {
                g0 = 0.25 * ((double)(a10[k] - a00[k]) * Dym + (double)(a11[k] - a01[k]) * Dy);
                g1 = 0.25 * ((double)(a01[k] - a00[k]) * Dxm + (double)(a11[k] - a10[k]) * Dx);
            }
            u0[t] = (float)g0;
            u1[t] = (float)g1;
        }
        dW[(int64_t)c * P + p] = make_float4(u0[0], u0[1], u0[2], u0[3]);
        dW[(int64_t)(NV + c) * P + p] = make_float4(u1[0], u1[1], u1[2], u1[3]);
    }
    for (int a = 0; a < 3; ++a) drg[(int64_t)a * P + p].w = (float)di0[a];
    dW[(int64_t)(2 * NV) * P + p] = make_float4((float)di1[0], (float)di1[1], (float)di1[2], 0.0f);
}

cudaError_t launch_geom_derivs(const ebsd_geometry& g, const int32_t* accum_e, int nE, int nsx,
                               int nsy, int e0, int nsel, int NV, float4* drg, float4* dW,
                               cudaStream_t s)
{
    WeightsGeom gd;
    const double dtor = (double)0.0174533f;
    const double alp =
        0.5 * 3.141592653589793238 - ((double)(float)g.sig - (double)g.thetac) * dtor;
    gd.L = g.L;
    gd.delta = g.delta;
    gd.xpc = g.xpc;
    gd.ypc = g.ypc;
    gd.ca = cos(alp);
    gd.sa = sin(alp);
    gd.numsx = g.numsx;
    gd.numsy = g.numsy;
    const int P = g.numsx * g.numsy;
    const int bs = 128;
    k_geom_derivs<<<(P + bs - 1) / bs, bs, 0, s>>>(gd, accum_e, nE, nsx, nsy, e0, nsel, NV, drg,
                                                   dW, P);
    return cudaGetLastError();
}

}  // namespace ebsd
