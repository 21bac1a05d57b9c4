/*
 * ebsd_oracle.c -- CPU restatement of the CTEMsoft CTEMEBSD pattern loop.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker for the GPU library:
 * only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may
 * load it.  The product (ctemsoft_gb300/, libebsdgpu.so) never links it.
 *
 * PARITY UNPINNED: the reference ships no tests, golden vectors or data for
 * this path, and it is Fortran-90 with no Fortran compiler available, so it
 * cannot be run to produce fixtures.  This restatement is pinned instead by
 * analytic known-answer tests (tests/test_oracle_kat.py) and by its own FP64
 * re-evaluation.
 *
 * Semantics mirrored (gfortran on x86-64, flags -O3 without -march/-ffast-math,
 * reference CMakeLists.txt:101-103): every real(sgl) operation is one IEEE
 * binary32 operation evaluated left to right, with no FMA contraction (this
 * file must be compiled with -ffp-contract=off); mixed sgl/dbl expressions are
 * promoted to binary64 and rounded once on assignment; int() truncates
 * toward zero; nint() rounds half away from zero; real**2 is x*x; the real
 * intrinsics sqrt, cos, sin, atan and real power map to libm sqrtf, cosf,
 * sinf, atanf and powf.
 *
 * Array conventions follow the Fortran declarations, first index fastest:
 *   rg[x + numsx*y]                    rgx/rgy/rgz(numsx,numsy)
 *   W[k + nE*(x + numsx*y)]            accum_e_detector(numEbins,numsx,numsy)
 *   accum_e[k + nE*(ix + (2nsx+1)*iy)] accum_e(numEbins,-nsx:nsx,-nsy:nsy)
 *   sr[ix + (2npx+1)*(iy + (2npy+1)*k)] sr(-npx:npx,-npy:npy,nE)
 *   pattern[x + numsx*y]               EBSDpattern(numsx,numsy)
 *
 * Documented divergences from the reference (both are undefined behaviour in
 * the Fortran and occur only at float rounding distance from a grid edge or
 * for non-divisible binning):
 *   - a bilinear corner index beyond the last grid node (nix+1 > npx or
 *     niy+1 > npy, CTEMEBSD.f90:504-506,601-603 read past the array) is
 *     clamped to the last node (edge replication);
 *   - accum_e_detector bins outside [Emin,Emax] (never written by
 *     CTEMEBSD.f90:502-507, yet summed at :516) are zero, which is what a
 *     fresh large allocation holds in practice;
 *   - binning crops to floor(numsx/b) x floor(numsy/b) full blocks
 *     (CTEMEBSD.f90:634-638 reads and writes past the arrays otherwise).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "ebsd_oracle.h"

/* CTEMEBSD.f90:150 -- the truncated degree-to-radian factor, kind sgl. */
#define DTOR_F 0.0174533f
/* Lambert.f90:239 dpi = 4*datan(1); constants.f90:70 cPi: the same binary64. */
static const double PI_D = 3.141592653589793238;

static double lps_spio2(void) { return sqrt(PI_D * 0.5); }       /* Lambert.f90:244 */
static double lps_spi2(void) { return sqrt(PI_D) * 0.5; }        /* Lambert.f90:243,245 */

/* ------------------------------------------------------------------ */
/* Lambert square <-> hemisphere                                       */
/* ------------------------------------------------------------------ */

/* Lambert.f90:405-436 Lambert2DSquareInverseSingle. */
int oracle_lambert_inverse_f32(const float xyz[3], float res[2])
{
    const float spi2 = (float)lps_spi2();               /* sngl(LPs%sPi2) */
    float s = xyz[0] * xyz[0];
    s = s + xyz[1] * xyz[1];
    s = s + xyz[2] * xyz[2];
    if (fabsf(1.0f - s) > 1.0e-6f) {                     /* :418 */
        res[0] = 0.0f; res[1] = 0.0f;
        return 1;
    }
    if (fabsf(xyz[2]) == 1.0f) {                          /* :423 */
        res[0] = 0.0f; res[1] = 0.0f;
    } else if (fabsf(xyz[1]) <= fabsf(xyz[0])) {          /* :426-428 */
        float q = fabsf(xyz[0]) / xyz[0] * sqrtf(2.0f * (1.0f - xyz[2]));
        res[0] = q * spi2;
        res[1] = q * atanf(xyz[1] / xyz[0]) / spi2;
    } else {                                              /* :430-431 */
        float q = fabsf(xyz[1]) / xyz[1] * sqrtf(2.0f * (1.0f - xyz[2]));
        res[0] = q * atanf(xyz[0] / xyz[1]) / spi2;
        res[1] = q * spi2;
    }
    return 0;
}

/* Lambert.f90:452-483 Lambert2DSquareInverseDouble. */
int oracle_lambert_inverse_f64(const double xyz[3], double res[2])
{
    const double spi2 = lps_spi2();
    double s = xyz[0] * xyz[0] + xyz[1] * xyz[1] + xyz[2] * xyz[2];
    if (fabs(1.0 - s) > 1.0e-12) {
        res[0] = 0.0; res[1] = 0.0;
        return 1;
    }
    if (fabs(xyz[2]) == 1.0) {
        res[0] = 0.0; res[1] = 0.0;
    } else if (fabs(xyz[1]) <= fabs(xyz[0])) {
        double q = fabs(xyz[0]) / xyz[0] * sqrt(2.0 * (1.0 - xyz[2]));
        res[0] = q * spi2;
        res[1] = q * atan(xyz[1] / xyz[0]) / spi2;
    } else {
        double q = fabs(xyz[1]) / xyz[1] * sqrt(2.0 * (1.0 - xyz[2]));
        res[0] = q * atan(xyz[0] / xyz[1]) / spi2;
        res[1] = q * spi2;
    }
    return 0;
}

/* Lambert.f90:352-389 Lambert2DSquareForwardDouble (Rosca 2010, eqs. 8-9).
 * Defines the master-grid convention: node (i,j) sits at (i,j)*sPio2/npx
 * (kvectors.f90:421-427,916-922). */
int oracle_lambert_forward_f64(const double xy[2], double res[3])
{
    const double spio2 = lps_spio2();
    const double ipi = 1.0 / PI_D;
    double ax = fabs(xy[0]), ay = fabs(xy[1]);
    double m = ax > ay ? ax : ay;
    if (m - spio2 > 1.0e-12) {
        res[0] = res[1] = res[2] = 0.0;
        return 1;
    }
    if (m == 0.0) {
        res[0] = 0.0; res[1] = 0.0; res[2] = 1.0;
    } else if (ax <= ay) {
        double q = 2.0 * xy[1] * ipi * sqrt(PI_D - xy[1] * xy[1]);
        double qq = xy[0] * PI_D * 0.25 / xy[1];
        res[0] = q * sin(qq);
        res[1] = q * cos(qq);
        res[2] = 1.0 - 2.0 * xy[1] * xy[1] * ipi;
    } else {
        double q = 2.0 * xy[0] * ipi * sqrt(PI_D - xy[0] * xy[0]);
        double qq = xy[1] * PI_D * 0.25 / xy[0];
        res[0] = q * cos(qq);
        res[1] = q * sin(qq);
        res[2] = 1.0 - 2.0 * xy[0] * xy[0] * ipi;
    }
    return 0;
}

/* ------------------------------------------------------------------ */
/* Quaternions and rotation conversions (scalar first)                 */
/* ------------------------------------------------------------------ */

/* quaternions.f90:255-264 quat_mult. */
void oracle_quat_mult_f32(const float x[4], const float y[4], float r[4])
{
    float r0 = x[0] * y[0] - x[1] * y[1] - x[2] * y[2] - x[3] * y[3];
    float r1 = x[0] * y[1] + x[1] * y[0] + x[2] * y[3] - x[3] * y[2];
    float r2 = x[0] * y[2] - x[1] * y[3] + x[2] * y[0] + x[3] * y[1];
    float r3 = x[0] * y[3] + x[1] * y[2] - x[2] * y[1] + x[3] * y[0];
    r[0] = r0; r[1] = r1; r[2] = r2; r[3] = r3;
}

static void quat_mult_f64(const double x[4], const double y[4], double r[4])
{
    double r0 = x[0] * y[0] - x[1] * y[1] - x[2] * y[2] - x[3] * y[3];
    double r1 = x[0] * y[1] + x[1] * y[0] + x[2] * y[3] - x[3] * y[2];
    double r2 = x[0] * y[2] - x[1] * y[3] + x[2] * y[0] + x[3] * y[1];
    double r3 = x[0] * y[3] + x[1] * y[2] - x[2] * y[1] + x[3] * y[0];
    r[0] = r0; r[1] = r1; r[2] = r2; r[3] = r3;
}

/* rotations.f90:1322-1351 eu2qu (Euler angles in radians). */
void oracle_eu2qu_f32(const float e[3], float res[4])
{
    float ee0 = 0.5f * e[0], ee1 = 0.5f * e[1], ee2 = 0.5f * e[2];
    float cPhi = cosf(ee1);
    float sPhi = sinf(ee1);
    float cm = cosf(ee0 - ee2);
    float sm = sinf(ee0 - ee2);
    float cp = cosf(ee0 + ee2);
    float sp = sinf(ee0 + ee2);
    float q = cPhi * cp;
    if (q < 0.0f) {
        res[0] = -q; res[1] = sPhi * cm; res[2] = sPhi * sm; res[3] = cPhi * sp;
    } else {
        res[0] = q; res[1] = -(sPhi * cm); res[2] = -(sPhi * sm); res[3] = -(cPhi * sp);
    }
}

/* rotations.f90:2116-2124 ax2qu = om2qu(ax2om(a)), with ax2om :743-775 and
 * om2qu :1575-1604 (quat_norm quaternions.f90:351-360).  a = (axis, angle rad). */
void oracle_ax2qu_f32(const float a[4], float res[4])
{
    float om[3][3];
    float c = cosf(a[3]);
    float s = sinf(a[3]);
    float omc = 1.0f - c;
    for (int i = 0; i < 3; ++i) om[i][i] = a[i] * a[i] * omc + c;
    float q = omc * a[0] * a[1];
    om[0][1] = q + s * a[2];
    om[1][0] = q - s * a[2];
    q = omc * a[1] * a[2];
    om[1][2] = q + s * a[0];
    om[2][1] = q - s * a[0];
    q = omc * a[2] * a[0];
    om[2][0] = q + s * a[1];
    om[0][2] = q - s * a[1];

    float t;
    t = om[0][0] + om[1][1] + om[2][2] + 1.0f;
    res[0] = sqrtf(t) / 2.0f;
    t = fabsf(om[0][0] - om[1][1] - om[2][2] + 1.0f);
    res[1] = sqrtf(t) / 2.0f;
    t = fabsf(-om[0][0] + om[1][1] - om[2][2] + 1.0f);
    res[2] = sqrtf(t) / 2.0f;
    t = fabsf(-om[0][0] - om[1][1] + om[2][2] + 1.0f);
    res[3] = sqrtf(t) / 2.0f;
    if (om[2][1] - om[1][2] < 0.0f) res[1] = -res[1];
    if (om[0][2] - om[2][0] < 0.0f) res[2] = -res[2];
    if (om[1][0] - om[0][1] < 0.0f) res[3] = -res[3];
    float n = res[0] * res[0];
    n = n + res[1] * res[1];
    n = n + res[2] * res[2];
    n = n + res[3] * res[3];
    float inv = 1.0f / sqrtf(n);
    for (int i = 0; i < 4; ++i) res[i] = inv * res[i];
}

/* CTEMEBSD.f90:244-288: angle-file rows to quaternions.  mode 0 = 'eu'
 * (degrees, optional hkl +90 deg on phi1), 1 = 'qu' (copied).  If
 * axisangle[3] != 0, q <- ax2qu(axis, angle*dtor) (x) q. */
void oracle_angles_to_quats_f32(const float* rows, int64_t n, int mode, int hkl,
                                const float axisangle[4], float* quats)
{
    for (int64_t i = 0; i < n; ++i) {
        if (mode == 0) {
            float e[3] = {rows[3 * i], rows[3 * i + 1], rows[3 * i + 2]};
            if (hkl) e[0] = e[0] + 90.0f;
            float er[3] = {e[0] * DTOR_F, e[1] * DTOR_F, e[2] * DTOR_F};
            oracle_eu2qu_f32(er, quats + 4 * i);
        } else {
            memcpy(quats + 4 * i, rows + 4 * i, 4 * sizeof(float));
        }
    }
    if (axisangle[3] != 0.0f) {
        float a[4] = {axisangle[0], axisangle[1], axisangle[2], axisangle[3] * DTOR_F};
        float qax[4];
        oracle_ax2qu_f32(a, qax);
        for (int64_t i = 0; i < n; ++i) {
            float r[4];
            oracle_quat_mult_f32(qax, quats + 4 * i, r);
            memcpy(quats + 4 * i, r, sizeof r);
        }
    }
}

/* ------------------------------------------------------------------ */
/* Detector geometry, CTEMEBSD.f90:416-452                              */
/* ------------------------------------------------------------------ */

void oracle_detector_f32(const oracle_geometry* g, float* rgx, float* rgy, float* rgz)
{
    const int nx = g->numsx, ny = g->numsy;
    float* scin_x = (float*)malloc(sizeof(float) * (size_t)nx);
    float* scin_y = (float*)malloc(sizeof(float) * (size_t)ny);
    for (int i = 0; i < nx; ++i)                                       /* :418 */
        scin_x[i] = -((g->xpc - (1.0f - (float)nx) * 0.5f - (float)i) * g->delta);
    for (int j = 0; j < ny; ++j)                                       /* :419 */
        scin_y[j] = (g->ypc - (1.0f - (float)ny) * 0.5f - (float)j) * g->delta;

    float sig = (float)g->sig;                                         /* :345 */
    float t = (sig - g->thetac) * DTOR_F;
    float alp = (float)(0.5 * PI_D - (double)t);                       /* :422 */
    float ca = cosf(alp), sa = sinf(alp);                              /* :423-424 */

    float L = g->L, L2 = L * L;                                        /* :433 */
    for (int j = 0; j < ny; ++j) {
        float sx = L2 + scin_y[j] * scin_y[j];
        float Ls = ca * scin_y[j] + L * sa;
        float Lc = -(sa * scin_y[j]) + L * ca;
        for (int i = 0; i < nx; ++i) {
            float rhos = 1.0f / sqrtf(sx + scin_x[i] * scin_x[i]);
            size_t p = (size_t)i + (size_t)nx * (size_t)j;
            rgx[p] = Ls * rhos;
            rgy[p] = scin_x[i] * rhos;
            rgz[p] = Lc * rhos;
        }
    }
    for (size_t p = 0; p < (size_t)nx * (size_t)ny; ++p) {            /* :448-451 */
        float z = rgx[p] * rgx[p];
        z = z + rgy[p] * rgy[p];
        z = z + rgz[p] * rgz[p];
        z = sqrtf(z);
        rgx[p] = rgx[p] / z;
        rgy[p] = rgy[p] / z;
        rgz[p] = rgz[p] / z;
    }
    free(scin_x);
    free(scin_y);
}

void oracle_detector_f64(const oracle_geometry_d* g, double* rgx, double* rgy, double* rgz)
{
    const int nx = g->numsx, ny = g->numsy;
    const double dtor = (double)DTOR_F;
    const double L = g->L, delta = g->delta;
    double alp = 0.5 * PI_D - (g->sig - g->thetac) * dtor;
    double ca = cos(alp), sa = sin(alp);
    for (int j = 0; j < ny; ++j) {
        double sy = (g->ypc - (1.0 - ny) * 0.5 - j) * delta;
        double Ls = ca * sy + L * sa;
        double Lc = -sa * sy + L * ca;
        for (int i = 0; i < nx; ++i) {
            double sx = -(g->xpc - (1.0 - nx) * 0.5 - i) * delta;
            double rhos = 1.0 / sqrt(L * L + sy * sy + sx * sx);
            double x = Ls * rhos, y = sx * rhos, z = Lc * rhos;
            double n = sqrt(x * x + y * y + z * z);
            size_t p = (size_t)i + (size_t)nx * (size_t)j;
            rgx[p] = x / n; rgy[p] = y / n; rgz[p] = z / n;
        }
    }
}

/* ------------------------------------------------------------------ */
/* Monte-Carlo energy weights on the detector, CTEMEBSD.f90:476-516     */
/* ------------------------------------------------------------------ */

static inline int clampi(int v, int hi) { return v > hi ? hi : v; }

/* W has nE*numsx*numsy entries (k fastest).  Bins outside [Emin,Emax]
 * (1-based, inclusive) are zero.  Returns num_el = nint(sum(W)) with the
 * single-precision sequential sum of :516. */
int32_t oracle_mc_weights_f32(const oracle_geometry* g, const float* rgx, const float* rgy,
                              const float* rgz, const int32_t* accum_e, int nE, int nsx,
                              int nsy, int Emin, int Emax, float* W)
{
    const int nx = g->numsx, ny = g->numsy;
    const int gx = 2 * nsx + 1;
    const float scl = (float)((double)(float)nsx / lps_spio2());       /* :481 */
    memset(W, 0, sizeof(float) * (size_t)nE * nx * ny);
    for (int i = 0; i < nx; ++i) {
        for (int j = 0; j < ny; ++j) {
            size_t p = (size_t)i + (size_t)nx * (size_t)j;
            float dc[3] = {rgx[p], rgy[p], rgz[p]};
            if (dc[2] < 0.0f) { dc[0] = -dc[0]; dc[1] = -dc[1]; dc[2] = -dc[2]; }
            float res[2];
            oracle_lambert_inverse_f32(dc, res);
            float ixy0 = scl * res[0], ixy1 = scl * res[1];
            float x = ixy0;                                             /* :491-493 */
            ixy0 = ixy1;
            ixy1 = -x;
            int nix = (int)((float)nsx + ixy0) - nsx;                   /* :495-500 */
            int niy = (int)((float)nsy + ixy1) - nsy;
            float dx = ixy0 - (float)nix;
            float dy = ixy1 - (float)niy;
            float dxm = 1.0f - dx;
            float dym = 1.0f - dy;
            int ix0 = nix + nsx, iy0 = niy + nsy;
            int ix1 = clampi(ix0 + 1, 2 * nsx), iy1 = clampi(iy0 + 1, 2 * nsy);
            const int32_t* a00 = accum_e + (size_t)nE * ((size_t)ix0 + (size_t)gx * iy0);
            const int32_t* a10 = accum_e + (size_t)nE * ((size_t)ix1 + (size_t)gx * iy0);
            const int32_t* a01 = accum_e + (size_t)nE * ((size_t)ix0 + (size_t)gx * iy1);
            const int32_t* a11 = accum_e + (size_t)nE * ((size_t)ix1 + (size_t)gx * iy1);
            float* w = W + (size_t)nE * p;
            for (int k = Emin - 1; k <= Emax - 1; ++k) {                /* :502-507 */
                w[k] = (float)a00[k] * dxm * dym + (float)a10[k] * dx * dym +
                       (float)a01[k] * dxm * dy + (float)a11[k] * dx * dy;
            }
        }
    }
    size_t tot = (size_t)nE * nx * ny;
    float s = 0.0f;
    for (size_t t = 0; t < tot; ++t) {                                 /* :510 then :516 */
        W[t] = W[t] * 0.25f;
        s = s + W[t];
    }
    return (int32_t)lroundf(s);
}

/* FP64 re-evaluation of the weights (same clamping, bins outside zero).
 * Returns the binary64 sum of W. */
double oracle_mc_weights_f64(const oracle_geometry_d* g, const double* rgx, const double* rgy,
                             const double* rgz, const int32_t* accum_e, int nE, int nsx,
                             int nsy, int Emin, int Emax, double* W)
{
    const int nx = g->numsx, ny = g->numsy;
    const int gx = 2 * nsx + 1;
    const double scl = (double)nsx / lps_spio2();
    double s = 0.0;
    memset(W, 0, sizeof(double) * (size_t)nE * nx * ny);
    for (int i = 0; i < nx; ++i) {
        for (int j = 0; j < ny; ++j) {
            size_t p = (size_t)i + (size_t)nx * (size_t)j;
            double dc[3] = {rgx[p], rgy[p], rgz[p]};
            if (dc[2] < 0.0) { dc[0] = -dc[0]; dc[1] = -dc[1]; dc[2] = -dc[2]; }
            double res[2];
            oracle_lambert_inverse_f64(dc, res);
            double ixy0 = scl * res[1], ixy1 = -(scl * res[0]);
            int nix = (int)(nsx + ixy0) - nsx;
            int niy = (int)(nsy + ixy1) - nsy;
            double dx = ixy0 - nix, dy = ixy1 - niy;
            double dxm = 1.0 - dx, dym = 1.0 - dy;
            int ix0 = nix + nsx, iy0 = niy + nsy;
            int ix1 = clampi(ix0 + 1, 2 * nsx), iy1 = clampi(iy0 + 1, 2 * nsy);
            const int32_t* a00 = accum_e + (size_t)nE * ((size_t)ix0 + (size_t)gx * iy0);
            const int32_t* a10 = accum_e + (size_t)nE * ((size_t)ix1 + (size_t)gx * iy0);
            const int32_t* a01 = accum_e + (size_t)nE * ((size_t)ix0 + (size_t)gx * iy1);
            const int32_t* a11 = accum_e + (size_t)nE * ((size_t)ix1 + (size_t)gx * iy1);
            double* w = W + (size_t)nE * p;
            for (int k = Emin - 1; k <= Emax - 1; ++k) {
                w[k] = 0.25 * (a00[k] * dxm * dym + a10[k] * dx * dym + a01[k] * dxm * dy +
                               a11[k] * dx * dy);
                s += w[k];
            }
        }
    }
    return s;
}

/* CTEMEBSD.f90:545 prefactor = 0.25*nAmpere*beamcurrent*dwelltime*1e-15/num_el. */
double oracle_prefactor(double beamcurrent, double dwelltime, int32_t num_el)
{
    const double nAmpere = 6.241e18;                                   /* :151 */
    return 0.25 * nAmpere * beamcurrent * dwelltime * 1.0e-15 / (double)num_el;
}

/* CTEMEBSD.f90:361-367 energy window (1-based, clamped to [1,numEbins]). */
void oracle_energy_window(float energymin, float energymax, double Ehistmin, double Ebinsize,
                          int numEbins, int* Emin, int* Emax)
{
    int a = (int)lround(((double)energymin - Ehistmin) / Ebinsize) + 1;
    int b = (int)lround(((double)energymax - Ehistmin) / Ebinsize) + 1;
    if (a < 1) a = 1;
    if (a > numEbins) a = numEbins;
    if (b < 1) b = 1;
    if (b > numEbins) b = numEbins;
    *Emin = a;
    *Emax = b;
}

/* ------------------------------------------------------------------ */
/* The pattern loop, CTEMEBSD.f90:571-608 (noise step :611-615 omitted) */
/* ------------------------------------------------------------------ */

/* One pixel's rotated Lambert coordinates: CTEMEBSD.f90:584-591. */
static inline void pixel_ixy_f32(const float q[4], float rx, float ry, float rz, float scl,
                                 float* ixy0, float* ixy1)
{
    const float qq1[4] = {q[0], -q[1], -q[2], -q[3]};                  /* conjg :577 */
    const float qq[4] = {0.0f, rx, ry, rz};                            /* :584 */
    float t[4], qq3[4];
    oracle_quat_mult_f32(qq, qq1, t);                                  /* :585 */
    oracle_quat_mult_f32(q, t, qq3);
    float dc[3] = {qq3[1], qq3[2], qq3[3]};
    float s = dc[0] * dc[0];                                           /* :588 */
    s = s + dc[1] * dc[1];
    s = s + dc[2] * dc[2];
    s = sqrtf(s);
    dc[0] = dc[0] / s; dc[1] = dc[1] / s; dc[2] = dc[2] / s;
    if (dc[2] < 0.0f) { dc[0] = -dc[0]; dc[1] = -dc[1]; dc[2] = -dc[2]; }  /* :589 */
    float res[2];
    oracle_lambert_inverse_f32(dc, res);                               /* :591 */
    *ixy0 = scl * res[0];
    *ixy1 = scl * res[1];
}

float oracle_master_scale_f32(int npx)                                 /* :571 */
{
    return (float)((double)(float)npx / lps_spio2());
}

/* Per-pixel Lambert cells: nix/niy (grid index, -npx..npx) and ixy for
 * each orientation; arrays are [N][numsy][numsx]. */
void oracle_cells_f32(const oracle_geometry* g, const float* rgx, const float* rgy,
                      const float* rgz, const float* quats, int64_t N, int npx, int npy,
                      int32_t* nix_out, int32_t* niy_out, float* ixy0_out, float* ixy1_out)
{
    const size_t P = (size_t)g->numsx * g->numsy;
    const float scl = oracle_master_scale_f32(npx);
    for (int64_t o = 0; o < N; ++o) {
        for (size_t p = 0; p < P; ++p) {
            float a, b;
            pixel_ixy_f32(quats + 4 * o, rgx[p], rgy[p], rgz[p], scl, &a, &b);
            nix_out[o * P + p] = (int)((float)npx + a) - npx;
            niy_out[o * P + p] = (int)((float)npy + b) - npy;
            ixy0_out[o * P + p] = a;
            ixy1_out[o * P + p] = b;
        }
    }
}

static void one_pattern_f32(const oracle_geometry* g, const float* rgx, const float* rgy,
                            const float* rgz, const float* W, int nE, int Emin, int Emax,
                            const float* sr, int npx, int npy, const float q[4],
                            double prefactor, float* out)
{
    const int nx = g->numsx, ny = g->numsy;
    const size_t gx = (size_t)(2 * npx + 1), gy = (size_t)(2 * npy + 1);
    const float scl = oracle_master_scale_f32(npx);
    for (int i = 0; i < nx; ++i) {                                     /* :581-606 */
        for (int j = 0; j < ny; ++j) {
            size_t p = (size_t)i + (size_t)nx * (size_t)j;
            float ixy0, ixy1;
            pixel_ixy_f32(q, rgx[p], rgy[p], rgz[p], scl, &ixy0, &ixy1);
            int nix = (int)((float)npx + ixy0) - npx;                  /* :593-598 */
            int niy = (int)((float)npy + ixy1) - npy;
            float dx = ixy0 - (float)nix;
            float dy = ixy1 - (float)niy;
            float dxm = 1.0f - dx;
            float dym = 1.0f - dy;
            size_t ix0 = (size_t)(nix + npx), iy0 = (size_t)(niy + npy);
            size_t ix1 = (size_t)clampi((int)ix0 + 1, 2 * npx);
            size_t iy1 = (size_t)clampi((int)iy0 + 1, 2 * npy);
            const float* w = W + (size_t)nE * p;
            float acc = 0.0f;                                          /* :579 */
            for (int k = Emin - 1; k <= Emax - 1; ++k) {               /* :600-604 */
                size_t plane = (size_t)k * gx * gy;
                float s00 = sr[plane + ix0 + gx * iy0];
                float s10 = sr[plane + ix1 + gx * iy0];
                float s01 = sr[plane + ix0 + gx * iy1];
                float s11 = sr[plane + ix1 + gx * iy1];
                acc = acc + w[k] * (s00 * dxm * dym + s10 * dx * dym + s01 * dxm * dy +
                                    s11 * dx * dy);
            }
            out[p] = (float)(prefactor * (double)acc);                 /* :608 */
        }
    }
}

/* Patterns [N][numsy][numsx] for N orientations, prefactor applied, no
 * noise, no binning.  nthreads > 1 splits orientations over OpenMP threads
 * (each pattern is computed exactly as in the serial loop). */
void oracle_patterns_f32(const oracle_geometry* g, const float* rgx, const float* rgy,
                         const float* rgz, const float* W, int nE, int Emin, int Emax,
                         const float* sr, int npx, int npy, const float* quats, int64_t N,
                         double prefactor, float* out, int nthreads)
{
    const size_t P = (size_t)g->numsx * g->numsy;
#ifdef _OPENMP
    if (nthreads < 1) nthreads = 1;
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads)
#endif
    for (int64_t o = 0; o < N; ++o)
        one_pattern_f32(g, rgx, rgy, rgz, W, nE, Emin, Emax, sr, npx, npy, quats + 4 * o,
                        prefactor, out + (size_t)o * P);
    (void)nthreads;
}

/* FP64 re-evaluation of the loop: binary64 throughout, with the inputs
 * (master at its stored float values; geometry and quaternions in binary64). */
void oracle_patterns_f64(const oracle_geometry_d* g, const double* rgx, const double* rgy,
                         const double* rgz, const double* W, int nE, int Emin, int Emax,
                         const float* sr, int npx, int npy, const double* quats, int64_t N,
                         double prefactor, double* out, int nthreads)
{
    const int nx = g->numsx, ny = g->numsy;
    const size_t P = (size_t)nx * ny;
    const size_t gx = (size_t)(2 * npx + 1), gy = (size_t)(2 * npy + 1);
    const double scl = (double)npx / lps_spio2();
#ifdef _OPENMP
    if (nthreads < 1) nthreads = 1;
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads)
#endif
    for (int64_t o = 0; o < N; ++o) {
        const double q[4] = {quats[4 * o], quats[4 * o + 1], quats[4 * o + 2], quats[4 * o + 3]};
        const double qc[4] = {q[0], -q[1], -q[2], -q[3]};
        for (size_t p = 0; p < P; ++p) {
            const double v[4] = {0.0, rgx[p], rgy[p], rgz[p]};
            double t[4], r[4];
            quat_mult_f64(v, qc, t);
            quat_mult_f64(q, t, r);
            double n = sqrt(r[1] * r[1] + r[2] * r[2] + r[3] * r[3]);
            double dc[3] = {r[1] / n, r[2] / n, r[3] / n};
            if (dc[2] < 0.0) { dc[0] = -dc[0]; dc[1] = -dc[1]; dc[2] = -dc[2]; }
            double res[2];
            oracle_lambert_inverse_f64(dc, res);
            double ixy0 = scl * res[0], ixy1 = scl * res[1];
            int nix = (int)(npx + ixy0) - npx;
            int niy = (int)(npy + ixy1) - npy;
            double dx = ixy0 - nix, dy = ixy1 - niy;
            double dxm = 1.0 - dx, dym = 1.0 - dy;
            size_t ix0 = (size_t)(nix + npx), iy0 = (size_t)(niy + npy);
            size_t ix1 = (size_t)clampi((int)ix0 + 1, 2 * npx);
            size_t iy1 = (size_t)clampi((int)iy0 + 1, 2 * npy);
            const double* w = W + (size_t)nE * p;
            double acc = 0.0;
            for (int k = Emin - 1; k <= Emax - 1; ++k) {
                size_t plane = (size_t)k * gx * gy;
                acc += w[k] * (sr[plane + ix0 + gx * iy0] * dxm * dym +
                               sr[plane + ix1 + gx * iy0] * dx * dym +
                               sr[plane + ix0 + gx * iy1] * dxm * dy +
                               sr[plane + ix1 + gx * iy1] * dx * dy);
            }
            out[(size_t)o * P + p] = prefactor * acc;
        }
    }
    (void)nthreads;
}

/* ------------------------------------------------------------------ */
/* Binning and gamma, CTEMEBSD.f90:630-651                              */
/* ------------------------------------------------------------------ */

/* mode: 0 'not' (copy), 1 'lin', 2 'gam'.  Output is [biny][binx] with
 * binx = numsx/b, biny = numsy/b (full blocks only) for modes 1 and 2. */
void oracle_epilogue_f32(const float* pat, int numsx, int numsy, int binning, int mode,
                         float gammavalue, float* out)
{
    if (mode == 0) {
        memcpy(out, pat, sizeof(float) * (size_t)numsx * numsy);
        return;
    }
    const int b = binning;
    const int bx = numsx / b, by = numsy / b;
    if (b != 1) {
        const float fb = (float)b;
        const float bindx = 1.0f / (fb * fb);                           /* :526 */
        for (int J = 0; J < by; ++J)
            for (int I = 0; I < bx; ++I) {
                float s = 0.0f;                                         /* :636 sum() */
                for (int jj = 0; jj < b; ++jj)
                    for (int ii = 0; ii < b; ++ii)
                        s = s + pat[(size_t)(I * b + ii) + (size_t)numsx * (J * b + jj)];
                out[(size_t)I + (size_t)bx * J] = s * bindx;            /* :640 */
            }
    } else {
        memcpy(out, pat, sizeof(float) * (size_t)numsx * numsy);        /* :642 */
    }
    if (mode == 2) {                                                    /* :647-649 */
        for (size_t t = 0; t < (size_t)bx * by; ++t) out[t] = powf(out[t], gammavalue);
    }
}

void oracle_epilogue_f64(const double* pat, int numsx, int numsy, int binning, int mode,
                         double gammavalue, double* out)
{
    if (mode == 0) {
        memcpy(out, pat, sizeof(double) * (size_t)numsx * numsy);
        return;
    }
    const int b = binning;
    const int bx = numsx / b, by = numsy / b;
    for (int J = 0; J < by; ++J)
        for (int I = 0; I < bx; ++I) {
            double s = 0.0;
            for (int jj = 0; jj < b; ++jj)
                for (int ii = 0; ii < b; ++ii)
                    s += pat[(size_t)(I * b + ii) + (size_t)numsx * (J * b + jj)];
            s /= (double)b * (double)b;
            out[(size_t)I + (size_t)bx * J] = mode == 2 ? pow(s, gammavalue) : s;
        }
}

int oracle_max_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
