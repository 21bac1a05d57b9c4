/*
 * ebsd_oracle_so3.c -- CPU restatement of CTEMsoft's cubochoric sampling of
 * a Rodrigues fundamental zone (the orientation list of an EBSD dictionary).
 * TEST INFRASTRUCTURE ONLY (the checker for ebsd_sample_rfz).
 * PARITY UNPINNED: the reference has no caller, test or fixture for
 * SampleRFZ and cannot be compiled here; the restatement is checked by
 * round trips and analytic properties.
 *
 * Followed, all in binary64 as the reference (SampleRFZ passes real(dbl)
 * coordinates, so the generic cu2ro resolves to cu2ro_d):
 *   constants      Lambert.f90:231-284 (InitLambertParameters)
 *   cube -> ball   Lambert.f90:960-1030 (Lambert3DCubeForwardDouble)
 *   ball -> cube   Lambert.f90:1150-1235 (Lambert3DCubeInverseDouble)
 *   pyramid        Lambert.f90:1314-1365 (GetPyramidDouble)
 *   ho -> ro       rotations.f90:2584-2619 (ho2ro_d)
 *   ro -> qu       rotations.f90:2233-2242 = ax2qu_d(ro2ax_d):
 *                  ro2ax_d :1209-1229, ax2om_d :791-824, om2qu_d :1618-1647
 *   FZ tests       so3.f90:105-245 (insideCyclicFZ, insideDihedralFZ,
 *                  insideCubicFZ), FZ type/order tables so3.f90:73-74
 *   sampler        so3.f90:267-371 (SampleRFZ)
 * gfortran evaluates a*b/c as (a*b)/c, x**2 as x*x and sum() left to
 * right; no FMA (-ffp-contract=off).
 */
#include <math.h>
#include <stdint.h>
#include <string.h>

#include "ebsd_oracle.h"

/* Lambert.f90:246-280 */
typedef struct {
    double Pi, sPi, srt, ap, a, sc, beta, R1, r2, r22, pi12, pi8, prek, r24, pref, rvmax2;
    double BP[6];
} lps_t;

static lps_t lps(void)
{
    lps_t L;
    const double dpi = 4.0 * atan(1.0);
    L.Pi = dpi;
    L.sPi = sqrt(dpi);
    L.srt = sqrt(3.0) / 2.0;
    L.pref = sqrt(6.0 / dpi);
    L.a = pow(dpi, 5.0 / 6.0) / pow(6.0, 1.0 / 6.0);
    L.ap = pow(dpi, 2.0 / 3.0);
    L.sc = L.a / L.ap;
    L.beta = 0.5 * L.a;
    L.R1 = pow(3.0 * dpi / 4.0, 1.0 / 3.0);
    L.r2 = sqrt(2.0);
    L.r22 = sqrt(2.0) / 2.0;
    L.pi12 = dpi / 12.0;
    L.pi8 = tan(dpi / 8.0);
    L.prek = L.R1 * pow(2.0, 0.25) / L.beta;
    L.r24 = sqrt(24.0);
    {
        const double t = tan(179.999 * dpi / 2.0 / 180.0);
        L.rvmax2 = t * t;
    }
    L.BP[0] = 0.0;
    L.BP[1] = tan(dpi / 4.0);
    L.BP[2] = tan(dpi / 6.0);
    L.BP[3] = L.pi8;
    L.BP[4] = 0.0;
    L.BP[5] = tan(L.pi12);
    return L;
}

void oracle_so3_constants(double out[8])
{
    const lps_t L = lps();
    out[0] = 0.5 * L.ap;  /* cube semi-edge (so3.f90:288) */
    out[1] = L.sc;
    out[2] = L.R1;
    out[3] = L.prek;
    out[4] = L.pref;
    out[5] = L.rvmax2;
    out[6] = L.pi8;
    out[7] = L.srt;
}

/* Lambert.f90:1314-1365; 0 if no pyramid matched (NaN input). */
static int pyramid(const double x[3])
{
    if (fabs(x[0]) <= x[2] && fabs(x[1]) <= x[2]) return 1;
    if (fabs(x[0]) <= -x[2] && fabs(x[1]) <= -x[2]) return 2;
    if (fabs(x[2]) <= x[0] && fabs(x[1]) <= x[0]) return 3;
    if (fabs(x[2]) <= -x[0] && fabs(x[1]) <= -x[0]) return 4;
    if (fabs(x[0]) <= x[1] && fabs(x[2]) <= x[1]) return 5;
    if (fabs(x[0]) <= -x[1] && fabs(x[2]) <= -x[1]) return 6;
    return 0;
}

static double maxabs3(const double x[3])
{
    double m = fabs(x[0]);
    if (fabs(x[1]) > m) m = fabs(x[1]);
    if (fabs(x[2]) > m) m = fabs(x[2]);
    return m;
}

/* Lambert.f90:960-1030: cubochoric -> homochoric. */
int oracle_cu2ho_d(const double c[3], double res[3])
{
    const lps_t L = lps();
    const double edge = 0.5 * pow(3.141592653589793238, 2.0 / 3.0);
    if (maxabs3(c) > edge) {
        res[0] = res[1] = res[2] = 0.0;
        return 1;
    }
    const int p = pyramid(c);
    double s3[3];
    if (p == 3 || p == 4) {
        s3[0] = c[1]; s3[1] = c[2]; s3[2] = c[0];
    } else if (p == 5 || p == 6) {
        s3[0] = c[2]; s3[1] = c[0]; s3[2] = c[1];
    } else {
        s3[0] = c[0]; s3[1] = c[1]; s3[2] = c[2];
    }
    const double X[3] = {L.sc * s3[0], L.sc * s3[1], L.sc * s3[2]};
    double lam[3];
    if (maxabs3(X) == 0.0) {
        lam[0] = lam[1] = lam[2] = 0.0;
    } else if ((fabs(X[0]) > fabs(X[1]) ? fabs(X[0]) : fabs(X[1])) == 0.0) {
        lam[0] = 0.0;
        lam[1] = 0.0;
        lam[2] = L.pref * X[2];
    } else {
        double cc, ss, q, T1, T2;
        if (fabs(X[1]) <= fabs(X[0])) {
            cc = cos(L.pi12 * X[1] / X[0]);
            ss = sin(L.pi12 * X[1] / X[0]);
            q = L.prek * X[0] / sqrt(L.r2 - cc);
            T1 = (L.r2 * cc - 1.0) * q;
            T2 = L.r2 * ss * q;
        } else {
            cc = cos(L.pi12 * X[0] / X[1]);
            ss = sin(L.pi12 * X[0] / X[1]);
            q = L.prek * X[1] / sqrt(L.r2 - cc);
            T1 = L.r2 * ss * q;
            T2 = (L.r2 * cc - 1.0) * q;
        }
        cc = T1 * T1 + T2 * T2;
        ss = L.Pi * cc / (24.0 * (X[2] * X[2]));
        cc = L.sPi * cc / L.r24 / X[2];
        q = sqrt(1.0 - ss);
        lam[0] = T1 * q;
        lam[1] = T2 * q;
        lam[2] = L.pref * X[2] - cc;
    }
    if (p == 3 || p == 4) {
        res[0] = lam[2]; res[1] = lam[0]; res[2] = lam[1];
    } else if (p == 5 || p == 6) {
        res[0] = lam[1]; res[1] = lam[2]; res[2] = lam[0];
    } else {
        res[0] = lam[0]; res[1] = lam[1]; res[2] = lam[2];
    }
    return 0;
}

/* Lambert.f90:1150-1235: homochoric -> cubochoric. */
int oracle_ho2cu_d(const double h[3], double res[3])
{
    const lps_t L = lps();
    const double rs = sqrt(h[0] * h[0] + h[1] * h[1] + h[2] * h[2]);
    res[0] = res[1] = res[2] = 0.0;
    if (rs > L.R1) return 1;
    if (maxabs3(h) == 0.0) return 0;
    const int p = pyramid(h);
    double x3[3];
    if (p == 3 || p == 4) {
        x3[0] = h[1]; x3[1] = h[2]; x3[2] = h[0];
    } else if (p == 5 || p == 6) {
        x3[0] = h[2]; x3[1] = h[0]; x3[2] = h[1];
    } else {
        x3[0] = h[0]; x3[1] = h[1]; x3[2] = h[2];
    }
    double q = sqrt(2.0 * rs / (rs + fabs(x3[2])));
    const double x2[3] = {x3[0] * q, x3[1] * q, (fabs(x3[2]) / x3[2]) * rs / L.pref};
    const double qxy = x2[0] * x2[0] + x2[1] * x2[1];
    const double sx = x2[0] != 0.0 ? fabs(x2[0]) / x2[0] : 1.0;
    const double sy = x2[1] != 0.0 ? fabs(x2[1]) / x2[1] : 1.0;
    double T1, T2;
    if (fabs(x2[1]) <= fabs(x2[0])) {
        const double q2xy = qxy + x2[0] * x2[0];
        const double sq2xy = sqrt(q2xy);
        q = (L.beta / L.r2 / L.R1) * sqrt(q2xy * qxy / (q2xy - fabs(x2[0]) * sq2xy));
        const double ac = acos((x2[1] * x2[1] + fabs(x2[0]) * sq2xy) / L.r2 / qxy);
        T1 = q * sx;
        T2 = q * sy * ac / L.pi12;
    } else {
        const double qx2y = qxy + x2[1] * x2[1];
        const double sqx2y = sqrt(qx2y);
        q = (L.beta / L.r2 / L.R1) * sqrt(qx2y * qxy / (qx2y - fabs(x2[1]) * sqx2y));
        const double ac = acos((x2[0] * x2[0] + fabs(x2[1]) * sqx2y) / L.r2 / qxy);
        T1 = q * sx * ac / L.pi12;
        T2 = q * sy;
    }
    const double x1[3] = {T1 / L.sc, T2 / L.sc, x2[2] / L.sc};
    if (p == 3 || p == 4) {
        res[0] = x1[2]; res[1] = x1[0]; res[2] = x1[1];
    } else if (p == 5 || p == 6) {
        res[0] = x1[1]; res[1] = x1[2]; res[2] = x1[0];
    } else {
        res[0] = x1[0]; res[1] = x1[1]; res[2] = x1[2];
    }
    return 0;
}

/* rotations.f90:2584-2619 (fit coefficients :2596-2599, also LPs%tfit). */
static const double kTfit[7] = {-0.5000096149170321, -0.02486606148871731,
                                -0.004549381779362819, 0.0005118668366387526,
                                -0.0016500827333575548, 0.0007593352203388718,
                                -0.0002040422502566876};

void oracle_ho2ro_d(const double h[3], double res[3])
{
    const double hmag = h[0] * h[0] + h[1] * h[1] + h[2] * h[2];
    if (hmag == 0.0) {
        res[0] = res[1] = res[2] = 0.0;
        return;
    }
    double hm = hmag;
    const double sq = sqrt(hmag);
    const double hn[3] = {h[0] / sq, h[1] / sq, h[2] / sq};
    double s = kTfit[0] * hmag;
    for (int i = 1; i < 7; ++i) {
        hm = hm * hmag;
        s = s + kTfit[i] * hm;
    }
    s = tan(acos(1.0 + s));
    res[0] = hn[0] * s;
    res[1] = hn[1] * s;
    res[2] = hn[2] * s;
}

void oracle_cu2ro_d(const double c[3], double rod[3])
{
    double h[3];
    oracle_cu2ho_d(c, h);
    oracle_ho2ro_d(h, rod);
}

/* ro2qu_d = ax2qu_d(ro2ax_d(r)) = om2qu_d(ax2om_d(ro2ax_d(r))).  A zero
 * vector (which ro2ax_d turns into NaN) gives the identity here. */
void oracle_ro2qu_d(const double r[3], double q[4])
{
    double ta = sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
    if (ta == 0.0) {
        q[0] = 1.0;
        q[1] = q[2] = q[3] = 0.0;
        return;
    }
    const double angle = 2.0 * atan(ta);
    double a[3] = {r[0] / ta, r[1] / ta, r[2] / ta};
    ta = sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
    a[0] = a[0] / ta;
    a[1] = a[1] / ta;
    a[2] = a[2] / ta;
    /* ax2om_d, om[i][j] = res(i+1, j+1) */
    const double c = cos(angle), s = sin(angle), omc = 1.0 - c;
    double om[3][3];
    for (int i = 0; i < 3; ++i) om[i][i] = a[i] * a[i] * omc + c;
    double t = omc * a[0] * a[1];
    om[0][1] = t + s * a[2];
    om[1][0] = t - s * a[2];
    t = omc * a[1] * a[2];
    om[1][2] = t + s * a[0];
    om[2][1] = t - s * a[0];
    t = omc * a[2] * a[0];
    om[2][0] = t + s * a[1];
    om[0][2] = t - s * a[1];
    /* om2qu_d */
    q[0] = sqrt(fabs(om[0][0] + om[1][1] + om[2][2] + 1.0)) / 2.0;
    q[1] = sqrt(fabs(om[0][0] - om[1][1] - om[2][2] + 1.0)) / 2.0;
    q[2] = sqrt(fabs(-om[0][0] + om[1][1] - om[2][2] + 1.0)) / 2.0;
    q[3] = sqrt(fabs(-om[0][0] - om[1][1] + om[2][2] + 1.0)) / 2.0;
    if (om[2][1] - om[1][2] < 0.0) q[1] = -q[1];
    if (om[0][2] - om[2][0] < 0.0) q[2] = -q[2];
    if (om[1][0] - om[0][1] < 0.0) q[3] = -q[3];
    const double n = 1.0 / sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3]);
    for (int i = 0; i < 4; ++i) q[i] = n * q[i];
}

/* so3.f90:73-74 */
static const int kFZtype[32] = {0, 0, 1, 1, 1, 2, 2, 2, 1, 1, 1, 2, 2, 2, 2, 1,
                                1, 2, 2, 2, 1, 1, 1, 2, 2, 2, 2, 3, 3, 4, 3, 4};
static const int kFZorder[32] = {0, 0, 2, 2, 2, 2, 2, 2, 4, 4, 4, 4, 4, 4, 4, 3,
                                 3, 3, 3, 3, 6, 6, 6, 6, 6, 6, 6, 0, 0, 0, 0, 0};

int oracle_fz_type(int pgnum, int* order)
{
    if (pgnum < 1 || pgnum > 32) return -1;
    if (order) *order = kFZorder[pgnum - 1];
    return kFZtype[pgnum - 1];
}

/* One point of SampleRFZ's loop body: 1 or 0 when the body assigns
 * insideFZ, 2 when it leaves the previous value (FZ types 0 and 1 with
 * |rod|^2 >= rvmax2 or NaN; so3.f90:335-340). */
int oracle_fz_code(const double rod[3], int type, int order)
{
    const lps_t L = lps();
    const double rx = rod[0], ry = rod[1], rz = rod[2];
    switch (type) {
        case 0: {
            const double rval = rx * rx + ry * ry + rz * rz;
            return rval < L.rvmax2 ? 1 : 2;
        }
        case 1: {
            const double rval = rx * rx + ry * ry + rz * rz;
            if (!(rval < L.rvmax2)) return 2;
            return fabs(rz) <= L.BP[order - 1] ? 1 : 0;  /* so3.f90:123-124 */
        }
        case 2: {  /* so3.f90:149-181 */
            if (!(fabs(rz) <= L.BP[order - 1])) return 0;
            int c2 = 0;
            switch (order) {
                case 2: c2 = fabs(rx) <= 1.0 && fabs(ry) <= 1.0; break;
                case 3:
                    c2 = fabs(L.srt * rx + 0.5 * ry) <= 1.0;
                    c2 = c2 && fabs(L.srt * rx - 0.5 * ry) <= 1.0;
                    c2 = c2 && fabs(ry) <= 1.0;
                    break;
                case 4:
                    c2 = fabs(rx) <= 1.0 && fabs(ry) <= 1.0;
                    c2 = c2 && (L.r22 * fabs(rx + ry) <= 1.0 && L.r22 * fabs(rx - ry) <= 1.0);
                    break;
                case 6:
                    c2 = fabs(0.5 * rx + L.srt * ry) <= 1.0;
                    c2 = c2 && fabs(L.srt * rx + 0.5 * ry) <= 1.0;
                    c2 = c2 && fabs(L.srt * rx - 0.5 * ry) <= 1.0;
                    c2 = c2 && fabs(0.5 * rx - L.srt * ry) <= 1.0;
                    c2 = c2 && fabs(ry) <= 1.0;
                    c2 = c2 && fabs(rx) <= 1.0;
                    break;
                default: c2 = 0;
            }
            return c2 ? 1 : 0;
        }
        default: {  /* 3 'tet', 4 'oct': so3.f90:215-244 */
            int c1 = 1;
            if (type == 4) c1 = maxabs3(rod) <= L.pi8;
            int c2 = fabs(rx + ry + rz) <= 1.0;
            c2 = c2 && fabs(-rx + ry + rz) <= 1.0;
            c2 = c2 && fabs(rx - ry + rz) <= 1.0;
            c2 = c2 && fabs(rx + ry - rz) <= 1.0;
            return (c1 && c2) ? 1 : 0;
        }
    }
}

/* The grid coordinates of SampleRFZ: x = -s, then x = x + delta while
 * x < s (so3.f90:288-291,316-368), accumulated in binary64. */
int64_t oracle_rfz_axis(int nsteps, double* xs, int64_t cap)
{
    const lps_t L = lps();
    const double s = 0.5 * L.ap;
    const double delta = s / (double)nsteps;
    int64_t m = 0;
    for (double x = -s; x < s; x = x + delta) {
        if (xs && m < cap) xs[m] = x;
        ++m;
    }
    return m;
}

/* SampleRFZ (so3.f90:267-371): Rodrigues vectors of the grid points inside
 * the FZ of point group pgnum, in loop order (x outer, z inner).  insideFZ
 * is never reset inside the loop; its value before the first assignment
 * is taken as .FALSE.  Returns the number of points (rods written up to
 * cap), or -1 for a bad point group / step count. */
int64_t oracle_sample_rfz(int nsteps, int pgnum, double* rods, int64_t cap)
{
    int order = 0;
    const int type = oracle_fz_type(pgnum, &order);
    if (type < 0 || nsteps < 1) return -1;
    const int64_t m = oracle_rfz_axis(nsteps, 0, 0);
    double xs[m > 0 ? m : 1];
    oracle_rfz_axis(nsteps, xs, m);
    int inside = 0;
    int64_t cnt = 0;
    for (int64_t i = 0; i < m; ++i)
        for (int64_t j = 0; j < m; ++j)
            for (int64_t k = 0; k < m; ++k) {
                const double c[3] = {xs[i], xs[j], xs[k]};
                double rod[3];
                oracle_cu2ro_d(c, rod);
                const int code = oracle_fz_code(rod, type, order);
                if (code != 2) inside = code;
                if (inside) {
                    if (rods && cnt < cap) memcpy(rods + 3 * cnt, rod, sizeof rod);
                    ++cnt;
                }
            }
    return cnt;
}
