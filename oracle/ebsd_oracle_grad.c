/*
 * ebsd_oracle_grad.c -- analytic FP64 derivatives of the EBSD pattern loop.
 *
 * TEST INFRASTRUCTURE ONLY (the checker for the GPU adjoint).  The
 * reference has no derivatives; this file differentiates the binary64
 * re-evaluation of CTEMEBSD.f90:416-608 (ebsd_oracle.c) by hand, in
 * forward mode, per pixel:
 *
 *   P(p) = prefactor * sum_k W_k(p) * B_k(ixy(p))
 *
 * where B_k is the bilinear master value of bin k (CTEMEBSD.f90:600-604),
 * ixy the scaled Lambert point of the rotated, normalised and folded
 * detector direction (:584-591, Lambert.f90:452-483), and W_k the
 * Monte-Carlo weight of the pixel (:483-510), itself a function of the
 * detector geometry.  Parameters: the left rotation tangent w, q(w) =
 * exp(w) (x) q with exp(w) = (cos|w|/2, sin(|w|/2) w/|w|), so that
 * d(direction)/dw_a = e_a x direction; and the pattern centre (xpc, ypc) in
 * pixels and L in microns.  The cell indices are locally constant, so
 * derivatives flow through the bilinear fractions only.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "ebsd_oracle.h"

static const double PI_D = 3.141592653589793238;
#define DTOR_D ((double)0.0174533f)

typedef struct {
    double X, Y;
    double dX[3], dY[3];
} lam_t;

/* Lambert2DSquareInverseDouble value and its Jacobian with respect to the
 * three components of the (unit, z >= 0) input vector. */
static void lambert_jac(const double v[3], lam_t* L)
{
    const double spi2 = sqrt(PI_D) * 0.5;
    const double x = v[0], y = v[1], z = v[2];
    memset(L, 0, sizeof *L);
    const double s = x * x + y * y + z * z;
    if (fabs(1.0 - s) > 1.0e-12 || fabs(z) == 1.0) return;
    const double rxy = x * x + y * y;
    const double rho = sqrt(2.0 * (1.0 - z));
    if (fabs(y) <= fabs(x)) {
        const double sg = fabs(x) / x;
        const double a = atan(y / x);
        L->X = sg * rho * spi2;
        L->Y = sg * rho * a / spi2;
        L->dX[2] = -sg * spi2 / rho;
        L->dY[0] = sg * rho / spi2 * (-y / rxy);
        L->dY[1] = sg * rho / spi2 * (x / rxy);
        L->dY[2] = -sg * a / (spi2 * rho);
    } else {
        const double sg = fabs(y) / y;
        const double b = atan(x / y);
        L->X = sg * rho * b / spi2;
        L->Y = sg * rho * spi2;
        L->dX[0] = sg * rho / spi2 * (y / rxy);
        L->dX[1] = sg * rho / spi2 * (-x / rxy);
        L->dX[2] = -sg * b / (spi2 * rho);
        L->dY[2] = -sg * spi2 / rho;
    }
}

static void qmul(const double x[4], const double y[4], double r[4])
{
    r[0] = x[0] * y[0] - x[1] * y[1] - x[2] * y[2] - x[3] * y[3];
    r[1] = x[0] * y[1] + x[1] * y[0] + x[2] * y[3] - x[3] * y[2];
    r[2] = x[0] * y[2] - x[1] * y[3] + x[2] * y[0] + x[3] * y[1];
    r[3] = x[0] * y[3] + x[1] * y[2] - x[2] * y[1] + x[3] * y[0];
}

static inline int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

/* Cell of CTEMEBSD.f90:593-598 in binary64: returns the 0-based lower
 * grid index (clamped) and the fraction. */
static int cell(double ixy, int np, double* d)
{
    const int ni = (int)((double)np + ixy) - np;
    *d = ixy - (double)ni;
    return clampi(ni + np, 0, 2 * np);
}

typedef struct {
    double rg[3];
    double drg[3][3]; /* d rg / d(xpc, ypc, L) */
} geom_t;

static void pixel_geometry(const oracle_geometry_d* g, int i, int j, double ca, double sa,
                           geom_t* out)
{
    const double sx = -(g->xpc - (1.0 - g->numsx) * 0.5 - i) * g->delta;
    const double sy = (g->ypc - (1.0 - g->numsy) * 0.5 - j) * g->delta;
    const double v[3] = {ca * sy + g->L * sa, sx, -sa * sy + g->L * ca};
    const double nv = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    for (int c = 0; c < 3; ++c) out->rg[c] = v[c] / nv;
    const double dv[3][3] = {{0.0, -g->delta, 0.0}, {ca * g->delta, 0.0, -sa * g->delta},
                             {sa, 0.0, ca}};
    for (int a = 0; a < 3; ++a) {
        const double pr = out->rg[0] * dv[a][0] + out->rg[1] * dv[a][1] + out->rg[2] * dv[a][2];
        for (int c = 0; c < 3; ++c) out->drg[a][c] = (dv[a][c] - pr * out->rg[c]) / nv;
    }
}

/* Weights W_k (window bins) and dW_k/d(xpc, ypc, L) of one pixel. */
static void pixel_weights(const geom_t* gm, const int32_t* acc, int nE, int nsx, int nsy,
                          int e0, int nsel, double* W, double* dW /* [3][nsel] */)
{
    double dc[3] = {gm->rg[0], gm->rg[1], gm->rg[2]};
    double sm = 1.0;
    if (dc[2] < 0.0) {
        dc[0] = -dc[0];
        dc[1] = -dc[1];
        dc[2] = -dc[2];
        sm = -1.0;
    }
    lam_t L;
    lambert_jac(dc, &L);
    const double scl = (double)nsx / sqrt(PI_D * 0.5);
    const double i0 = scl * L.Y, i1 = -(scl * L.X); /* swap, CTEMEBSD.f90:491-493 */
    double Dx, Dy;
    const int jx0 = cell(i0, nsx, &Dx), jy0 = cell(i1, nsy, &Dy);
    const int jx1 = clampi(jx0 + 1, 0, 2 * nsx), jy1 = clampi(jy0 + 1, 0, 2 * nsy);
    const double Dxm = 1.0 - Dx, Dym = 1.0 - Dy;
    const size_t gx = (size_t)(2 * nsx + 1);
    const int32_t* a00 = acc + ((size_t)jy0 * gx + jx0) * nE + e0;
    const int32_t* a10 = acc + ((size_t)jy0 * gx + jx1) * nE + e0;
    const int32_t* a01 = acc + ((size_t)jy1 * gx + jx0) * nE + e0;
    const int32_t* a11 = acc + ((size_t)jy1 * gx + jx1) * nE + e0;
    double di0[3], di1[3]; /* d i0 / d theta_a, d i1 / d theta_a */
    for (int a = 0; a < 3; ++a) {
        double t0 = 0.0, t1 = 0.0;
        for (int c = 0; c < 3; ++c) {
            t0 += scl * sm * L.dY[c] * gm->drg[a][c];
            t1 += -scl * sm * L.dX[c] * gm->drg[a][c];
        }
        di0[a] = t0;
        di1[a] = t1;
    }
    for (int k = 0; k < nsel; ++k) {
        W[k] = 0.25 * (a00[k] * Dxm * Dym + a10[k] * Dx * Dym + a01[k] * Dxm * Dy +
                       a11[k] * Dx * Dy);
        const double g0 = 0.25 * ((a10[k] - a00[k]) * Dym + (a11[k] - a01[k]) * Dy);
        const double g1 = 0.25 * ((a01[k] - a00[k]) * Dxm + (a11[k] - a10[k]) * Dx);
        for (int a = 0; a < 3; ++a) dW[a * nsel + k] = g0 * di0[a] + g1 * di1[a];
    }
}

/* Value and 6 derivatives (w0,w1,w2,xpc,ypc,L) of one pixel. */
static double pixel_value(const geom_t* gm, const double* W, const double* dW, int nsel,
                          const float* sr, int e0, int npx, int npy, const double q[4],
                          double prefactor, double J[6])
{
    const double qc[4] = {q[0], -q[1], -q[2], -q[3]};
    const double v[4] = {0.0, gm->rg[0], gm->rg[1], gm->rg[2]};
    double t[4], r[4];
    qmul(v, qc, t);
    qmul(q, t, r);
    const double d[3] = {r[1], r[2], r[3]};
    const double nd = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
    double dh[3] = {d[0] / nd, d[1] / nd, d[2] / nd};
    double s = 1.0;
    double dc[3] = {dh[0], dh[1], dh[2]};
    if (dc[2] < 0.0) {
        s = -1.0;
        dc[0] = -dc[0];
        dc[1] = -dc[1];
        dc[2] = -dc[2];
    }
    lam_t L;
    lambert_jac(dc, &L);
    const double scl = (double)npx / sqrt(PI_D * 0.5);
    double dx, dy;
    const int ix0 = cell(scl * L.X, npx, &dx), iy0 = cell(scl * L.Y, npy, &dy);
    const int ix1 = clampi(ix0 + 1, 0, 2 * npx), iy1 = clampi(iy0 + 1, 0, 2 * npy);
    const double dxm = 1.0 - dx, dym = 1.0 - dy;
    const size_t gx = (size_t)(2 * npx + 1), plane = gx * (size_t)(2 * npy + 1);
    double P = 0.0, gX = 0.0, gY = 0.0, gW[3] = {0.0, 0.0, 0.0};
    for (int k = 0; k < nsel; ++k) {
        const float* m = sr + (size_t)(e0 + k) * plane;
        const double s00 = m[(size_t)iy0 * gx + ix0], s10 = m[(size_t)iy0 * gx + ix1];
        const double s01 = m[(size_t)iy1 * gx + ix0], s11 = m[(size_t)iy1 * gx + ix1];
        const double B = s00 * dxm * dym + s10 * dx * dym + s01 * dxm * dy + s11 * dx * dy;
        P += W[k] * B;
        gX += W[k] * ((s10 - s00) * dym + (s11 - s01) * dy);
        gY += W[k] * ((s01 - s00) * dxm + (s11 - s10) * dx);
        for (int a = 0; a < 3; ++a) gW[a] += dW[a * nsel + k] * B;
    }
    double gdc[3], gd[3];
    for (int c = 0; c < 3; ++c) gdc[c] = scl * (gX * L.dX[c] + gY * L.dY[c]);
    const double pr = gdc[0] * dh[0] + gdc[1] * dh[1] + gdc[2] * dh[2];
    for (int c = 0; c < 3; ++c) gd[c] = s * (gdc[c] - pr * dh[c]) / nd;
    /* rotation tangent: d/dw_a of P = gd . (e_a x d) = (d x gd)_a */
    J[0] = prefactor * (d[1] * gd[2] - d[2] * gd[1]);
    J[1] = prefactor * (d[2] * gd[0] - d[0] * gd[2]);
    J[2] = prefactor * (d[0] * gd[1] - d[1] * gd[0]);
    /* pattern centre: (M^T gd) . drg_a + dW_a terms, M^T gd = conj(q) (x) gd (x) q */
    const double gv[4] = {0.0, gd[0], gd[1], gd[2]};
    double u[4], w[4];
    qmul(gv, q, u);
    qmul(qc, u, w);
    for (int a = 0; a < 3; ++a)
        J[3 + a] = prefactor * (w[1] * gm->drg[a][0] + w[2] * gm->drg[a][1] +
                                w[3] * gm->drg[a][2] + gW[a]);
    return prefactor * P;
}

void oracle_vjp_f64(const oracle_geometry_d* g, const int32_t* accum_e, int nE, int nsx, int nsy,
                    int Emin, int Emax, const float* sr, int npx, int npy, const double* quats,
                    int64_t N, double prefactor, int binning, int mode, const float* data,
                    double* loss, double* grad, int nthreads)
{
    const int nx = g->numsx, ny = g->numsy;
    const int e0 = Emin - 1, nsel = Emax - Emin + 1;
    const int b = binning < 1 ? 1 : binning;
    const int ox = nx / b, oy = ny / b;
    const size_t P = (size_t)nx * ny, OUT = (size_t)ox * oy;
    const double alp = 0.5 * PI_D - (g->sig - g->thetac) * DTOR_D;
    const double ca = cos(alp), sa = sin(alp);
    geom_t* gm = (geom_t*)malloc(sizeof(geom_t) * P);
    double* W = (double*)malloc(sizeof(double) * P * nsel);
    double* dW = (double*)malloc(sizeof(double) * P * 3 * nsel);
    for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) {
            const size_t p = (size_t)j * nx + i;
            pixel_geometry(g, i, j, ca, sa, &gm[p]);
            pixel_weights(&gm[p], accum_e, nE, nsx, nsy, e0, nsel, W + p * nsel,
                          dW + p * 3 * nsel);
        }
    const double ib2 = 1.0 / ((double)b * (double)b);
#ifdef _OPENMP
    if (nthreads < 1) nthreads = 1;
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads)
#endif
    for (int64_t n = 0; n < N; ++n) {
        double* O = (double*)calloc(OUT * 7, sizeof(double)); /* value + 6 derivatives */
        for (int j = 0; j < oy * b; ++j)
            for (int i = 0; i < ox * b; ++i) {
                const size_t p = (size_t)j * nx + i;
                double J[6];
                const double v = pixel_value(&gm[p], W + p * nsel, dW + p * 3 * nsel, nsel, sr,
                                             e0, npx, npy, quats + 4 * n, prefactor, J);
                double* o = O + 7 * ((size_t)(j / b) * ox + i / b);
                o[0] += v * ib2;
                for (int a = 0; a < 6; ++a) o[1 + a] += J[a] * ib2;
            }
        const float* d = data + (size_t)n * OUT;
        double G[6] = {0, 0, 0, 0, 0, 0};
        if (mode == 0) {
            for (size_t B = 0; B < OUT; ++B)
                for (int a = 0; a < 6; ++a) G[a] += (double)d[B] * O[7 * B + 1 + a];
            if (loss) loss[n] = 0.0;
        } else {
            double soo = 0, sot = 0, stt = 0, ST[6] = {0}, SO[6] = {0};
            for (size_t B = 0; B < OUT; ++B) {
                const double o = O[7 * B], t = d[B];
                soo += o * o;
                sot += o * t;
                stt += t * t;
                for (int a = 0; a < 6; ++a) {
                    ST[a] += t * O[7 * B + 1 + a];
                    SO[a] += o * O[7 * B + 1 + a];
                }
            }
            const double den = sqrt(soo * stt);
            for (int a = 0; a < 6; ++a) G[a] = -(ST[a] - sot / soo * SO[a]) / den;
            if (loss) loss[n] = 1.0 - sot / den;
        }
        memcpy(grad + 6 * n, G, sizeof G);
        free(O);
    }
    (void)nthreads;
    free(gm);
    free(W);
    free(dW);
}
