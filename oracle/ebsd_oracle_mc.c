/*
 * ebsd_oracle_mc.c -- CPU restatement of CTEMsoft's Monte-Carlo backscatter
 * histogram (CTEMMC.f90:307-529, single_run; CSDA mode).
 * TEST INFRASTRUCTURE ONLY (the checker for ebsd_mc_run).
 * PARITY UNPINNED: the reference has no tests or fixtures for CTEMMC and
 * cannot be compiled here.  (The Philox4x32-10 block below is pinned to the
 * known-answer vectors its authors publish; the trajectory physics is not.)
 *
 * Two random-number sources drive the same trajectory code:
 *   - the GPU's: Philox4x32-10 keyed by the seed, counter (draw/4, 0,
 *     electron), one 32-bit word per draw -- so the oracle and the GPU
 *     follow the same electrons draw for draw;
 *   - the reference's own (rng.f95: a lag-3 subtract generator modulo
 *     2147483579 plus the 69069 LCG, one stream per OpenMP thread seeded
 *     primeseed + i, CTEMMC.f90:226), for statistical comparison.
 * Both turn a 32-bit signed word w into u = real(0.5d0 + 0.23283064d-9*w)
 * (rng.f95), a single-precision value, as the reference does.
 *
 * Arithmetic is binary64 left to right as gfortran evaluates it
 * (-ffp-contract=off); literals without a D exponent (0.67, 1.166, 10.0)
 * are single precision, as in the reference source.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "ebsd_oracle.h"

typedef struct {
    double sig, omega, EkeV, Ehistmin, Ebinsize, depthmax, depthstep, Ze, density, at_wt;
    int numsx, nx, numEbins, numzbins, nz10;
    /* derived, CTEMMC.f90:410-440 */
    double Emin, pre, prealpha, J, predEds, tpi, tano, delta, cxstart, czstart, sPi2;
} mcs_t;

static const double kPi = 3.141592653589, kAvogadro = 6.0221415e+23, kDtoR = 0.017453293;
static const double kPresig = 1.5273987e19, kScaled = 1.0e8, kMinEnergy = 1.0;

int oracle_mc_dims(const oracle_mc_params* p, int* numEbins, int* numzbins)
{
    if (!(p->Ebinsize > 0.0) || !(p->depthstep > 0.0) || !(p->EkeV > p->Ehistmin) ||
        p->numsx < 3 || (p->numsx % 2) == 0)
        return -1;
    *numEbins = (int)((p->EkeV - p->Ehistmin) / p->Ebinsize) + 1;   /* CTEMMC.f90:205-206 */
    *numzbins = (int)(p->depthmax / p->depthstep) + 1;
    return 0;
}

static int setup(const oracle_mc_params* p, mcs_t* s)
{
    memset(s, 0, sizeof *s);
    s->sig = p->sig;
    s->omega = p->omega;
    s->EkeV = p->EkeV;
    s->Ehistmin = p->Ehistmin;
    s->Ebinsize = p->Ebinsize;
    s->depthmax = p->depthmax;
    s->depthstep = p->depthstep;
    s->Ze = p->Ze;
    s->density = p->density;
    s->at_wt = p->at_wt;
    s->numsx = p->numsx;
    if (oracle_mc_dims(p, &s->numEbins, &s->numzbins)) return -1;
    s->nx = (p->numsx - 1) / 2;
    s->nz10 = s->nx / 10;
    s->Emin = s->Ehistmin - s->Ebinsize / 2.0;
    s->pre = s->at_wt / kAvogadro / s->density;
    s->prealpha = 3.4e-3 * pow(s->Ze, (double)0.67f);
    double J = (9.76 * s->Ze + 58.5 / pow(s->Ze, 0.19)) * 1.0e-3 / (double)1.166f;
    s->J = 1.0 / J;
    s->predEds = -78500.0 * s->density * s->Ze / s->at_wt;
    s->tpi = 2.0 * kPi;
    s->tano = tan(s->omega * kDtoR);
    /* LPs%sPio2 = sqrt(pi/2), LPs%sPi2 = sqrt(pi)/2 with pi = 4 atan(1) */
    const double dpi = 4.0 * atan(1.0);
    s->delta = (double)s->nx / sqrt(dpi * 0.5);
    s->sPi2 = sqrt(dpi) * 0.5;
    s->cxstart = cos((90.0 - s->sig) * kDtoR);
    s->czstart = -sin((90.0 - s->sig) * kDtoR);
    return 0;
}

/* ---- random numbers ------------------------------------------------ */

static float u_from_word(uint32_t w)
{
    return (float)(0.5 + 0.23283064e-9 * (double)(int32_t)w);  /* rng.f95 */
}

/* Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11). */
static void philox(uint32_t c[4], uint32_t k0, uint32_t k1)
{
    for (int r = 0; r < 10; ++r) {
        const uint64_t p0 = (uint64_t)0xD2511F53u * c[0];
        const uint64_t p1 = (uint64_t)0xCD9E8D57u * c[2];
        const uint32_t n0 = (uint32_t)(p1 >> 32) ^ c[1] ^ k0;
        const uint32_t n2 = (uint32_t)(p0 >> 32) ^ c[3] ^ k1;
        c[0] = n0;
        c[1] = (uint32_t)p1;
        c[2] = n2;
        c[3] = (uint32_t)p0;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
}

/* One raw Philox4x32-10 block, exported so that the generator can be checked
 * against the published known-answer vectors of its authors. */
void oracle_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4])
{
    uint32_t c[4] = {ctr[0], ctr[1], ctr[2], ctr[3]};
    philox(c, key[0], key[1]);
    for (int i = 0; i < 4; ++i) out[i] = c[i];
}

typedef struct {
    int kind;  /* 0 Philox, 1 reference */
    /* Philox */
    uint32_t k0, k1, e_lo, e_hi, block;
    uint32_t buf[4];
    int pos;
    /* reference rng.f95 */
    int32_t st[4];
} rng_t;

static float next_u(rng_t* r)
{
    if (r->kind == 0) {
        if (r->pos == 4) {
            uint32_t c[4] = {r->block, 0u, r->e_lo, r->e_hi};
            philox(c, r->k0, r->k1);
            memcpy(r->buf, c, sizeof c);
            r->pos = 0;
            ++r->block;
        }
        return u_from_word(r->buf[r->pos++]);
    }
    int32_t imz = r->st[0] - r->st[2];
    if (imz < 0) imz += 2147483579;
    r->st[0] = r->st[1];
    r->st[1] = r->st[2];
    r->st[2] = imz;
    r->st[3] = (int32_t)(69069u * (uint32_t)r->st[3] + 1013904243u);  /* wraps like int32 */
    imz = (int32_t)((uint32_t)imz + (uint32_t)r->st[3]);
    return u_from_word((uint32_t)imz);
}

/* ---- one electron (CTEMMC.f90:444-524) ------------------------------ */

/* Lambert.f90:452-483, the binary64 square-Lambert inverse. */
static void sphere_to_square(const mcs_t* s, const double v[3], double res[2])
{
    const double n = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
    res[0] = res[1] = 0.0;
    if (fabs(1.0 - n) > 1.0e-12) return;
    if (fabs(v[2]) == 1.0) return;
    if (fabs(v[1]) <= fabs(v[0])) {
        const double q = fabs(v[0]) / v[0] * sqrt(2.0 * (1.0 - v[2]));
        res[0] = q * s->sPi2;
        res[1] = q * atan(v[1] / v[0]) / s->sPi2;
    } else {
        const double q = fabs(v[1]) / v[1] * sqrt(2.0 * (1.0 - v[2]));
        res[0] = q * atan(v[0] / v[1]) / s->sPi2;
        res[1] = q * s->sPi2;
    }
}

static void free_path(const mcs_t* s, double Ec, double* alpha, double* lambda)
{
    *alpha = s->prealpha / Ec;
    double step = Ec * (Ec + 1024.0) / s->Ze / (Ec + 511.0);
    const double sige = kPresig * step * step * *alpha * (1.0 + *alpha);
    *lambda = s->pre * sige;
}

/* Returns 1 if the electron was counted in accum_e. */
static int electron(const mcs_t* s, rng_t* r, int32_t* accum_e, int32_t* accum_z)
{
    double Ec = s->EkeV;
    double xyz[3] = {0.0, 0.0, 0.0};
    double alpha, lambda;
    free_path(s, Ec, &alpha, &lambda);
    double rr = (double)next_u(r);
    double step = -lambda * log(rr);
    double cxyz[3] = {s->cxstart, 0.0, s->czstart};
    for (int i = 0; i < 3; ++i) xyz[i] = xyz[i] + step * kScaled * cxyz[i];
    for (int traj = 0; traj < 5000; ++traj) {
        const double dEds = s->predEds * log(Ec * s->J + 1.0) / Ec;
        const double dE = dEds * step;
        Ec = Ec + dE;
        if (Ec < kMinEnergy) return 0;
        rr = (double)next_u(r);
        const double cphi = 1.0 - 2.0 * alpha * rr / (1.0 + alpha - rr);
        const double sphi = sin(acos(cphi));
        rr = (double)next_u(r);
        const double psi = s->tpi * rr;
        const double spsi = sin(psi), cpsi = cos(psi);
        double cp[3];
        if (fabs(cxyz[2]) > 0.99999) {
            cp[0] = sphi * cpsi;
            cp[1] = sphi * spsi;
            cp[2] = (cxyz[2] / fabs(cxyz[2])) * cphi;
        } else {
            const double dsq = sqrt(1.0 - cxyz[2] * cxyz[2]);
            const double dsqi = 1.0 / dsq;
            cp[0] = sphi * (cxyz[0] * cxyz[2] * cpsi - cxyz[1] * spsi) * dsqi + cxyz[0] * cphi;
            cp[1] = sphi * (cxyz[1] * cxyz[2] * cpsi + cxyz[0] * spsi) * dsqi + cxyz[1] * cphi;
            cp[2] = -(sphi * cpsi * dsq) + cxyz[2] * cphi;
        }
        const double dd = 1.0 / sqrt(cp[0] * cp[0] + cp[1] * cp[1] + cp[2] * cp[2]);
        for (int i = 0; i < 3; ++i) cp[i] = cp[i] * dd;
        free_path(s, Ec, &alpha, &lambda);
        rr = (double)next_u(r);
        step = -lambda * log(rr);
        double xn[3];
        for (int i = 0; i < 3; ++i) xn[i] = xyz[i] + step * kScaled * cp[i];
        const double znmax = xn[1] * s->tano;
        if (xn[2] > znmax) {
            double dxy[2];
            sphere_to_square(s, cp, dxy);
            dxy[0] = s->delta * dxy[0];
            dxy[1] = s->delta * dxy[1];
            if (!isfinite(dxy[0]) || !isfinite(dxy[1])) return 0;  /* NaN direction */
            const long ix = lround(dxy[1]), iy = lround(-dxy[0]);
            int counted = 0;
            if (labs(ix) <= s->nx && labs(iy) <= s->nx && Ec > s->Emin) {
                const long iE = lround((Ec - s->Ehistmin) / s->Ebinsize) + 1;
                if (iE >= 1 && iE <= s->numEbins) {  /* the reference does not check */
                    const double edis = fabs(xyz[2] / cp[2]);
                    const double zb = edis * 0.1 / s->depthstep;
                    const long iz = zb < 1.0e15 ? lround(zb) + 1 : -1;
                    if (iz > 0 && iz <= s->numzbins && accum_z) {
                        const long px = lroundf((float)ix / 10.0f);
                        const long py = lroundf((float)iy / 10.0f);
                        if (labs(px) <= s->nz10 && labs(py) <= s->nz10) {
                            const long w = 2 * s->nz10 + 1;
                            accum_z[(iE - 1) + (long)s->numEbins *
                                                   ((iz - 1) + (long)s->numzbins *
                                                                   ((px + s->nz10) + w * (py + s->nz10)))] += 1;
                        }
                    }
                    const long g = 2 * s->nx + 1;
                    accum_e[(iE - 1) + (long)s->numEbins * ((ix + s->nx) + g * (iy + s->nx))] += 1;
                    counted = 1;
                }
            }
            return counted;
        }
        for (int i = 0; i < 3; ++i) {
            cxyz[i] = cp[i];
            xyz[i] = xn[i];
        }
    }
    return 0;
}

/* Electrons [e0, e1) with the Philox stream of `seed`; accum arrays are
 * added to (accum_z may be NULL).  Returns the electrons counted. */
int64_t oracle_mc_philox(const oracle_mc_params* p, uint64_t seed, int64_t e0, int64_t e1,
                         int32_t* accum_e, int32_t* accum_z)
{
    mcs_t s;
    if (setup(p, &s)) return -1;
    int64_t n = 0;
    for (int64_t e = e0; e < e1; ++e) {
        rng_t r;
        memset(&r, 0, sizeof r);
        r.kind = 0;
        r.k0 = (uint32_t)seed;
        r.k1 = (uint32_t)(seed >> 32);
        r.e_lo = (uint32_t)e;
        r.e_hi = (uint32_t)((uint64_t)e >> 32);
        r.pos = 4;
        n += electron(&s, &r, accum_e, accum_z);
    }
    return n;
}

/* The reference's own streams: for i = 1..nthreads, rng_seed(primeseed+i),
 * then num_el electrons in sequence (CTEMMC.f90:224-237).  As in the
 * reference, each stream runs on its own OpenMP thread into private
 * histograms that are added at the end (the CRITICAL section of :234-237);
 * integer sums, so the result does not depend on the thread count. */
int64_t oracle_mc_reference_rng(const oracle_mc_params* p, int32_t primeseed, int nthreads,
                                int64_t num_el, int32_t* accum_e, int32_t* accum_z)
{
    mcs_t s;
    if (setup(p, &s)) return -1;
    const size_t ne = (size_t)s.numEbins * s.numsx * s.numsx;
    const size_t w10 = 2 * (size_t)s.nz10 + 1;
    const size_t nzs = (size_t)s.numEbins * s.numzbins * w10 * w10;
    int64_t n = 0;
#pragma omp parallel for schedule(static, 1) reduction(+ : n)
    for (int i = 1; i <= nthreads; ++i) {
        int32_t* ae = (int32_t*)calloc(ne, sizeof(int32_t));
        int32_t* az = accum_z ? (int32_t*)calloc(nzs, sizeof(int32_t)) : NULL;
        rng_t r;
        memset(&r, 0, sizeof r);
        r.kind = 1;
        r.st[0] = primeseed + i;
        r.st[1] = 362436069;
        r.st[2] = 16163801;
        r.st[3] = 1131199299;
        int64_t c = 0;
        if (ae && (az || !accum_z))
            for (int64_t e = 0; e < num_el; ++e) c += electron(&s, &r, ae, az);
#pragma omp critical
        {
            if (ae)
                for (size_t k = 0; k < ne; ++k) accum_e[k] += ae[k];
            if (az)
                for (size_t k = 0; k < nzs; ++k) accum_z[k] += az[k];
        }
        free(ae);
        free(az);
        n += c;
    }
    return n;
}

/* The random values themselves, for checking the generators. */
void oracle_mc_uniforms(int kind, uint64_t seed_or_prime, int64_t electron, int count, float* u)
{
    rng_t r;
    memset(&r, 0, sizeof r);
    r.kind = kind;
    if (kind == 0) {
        r.k0 = (uint32_t)seed_or_prime;
        r.k1 = (uint32_t)(seed_or_prime >> 32);
        r.e_lo = (uint32_t)electron;
        r.e_hi = (uint32_t)((uint64_t)electron >> 32);
        r.pos = 4;
    } else {
        r.st[0] = (int32_t)seed_or_prime;
        r.st[1] = 362436069;
        r.st[2] = 16163801;
        r.st[3] = 1131199299;
    }
    for (int i = 0; i < count; ++i) u[i] = next_u(&r);
}
