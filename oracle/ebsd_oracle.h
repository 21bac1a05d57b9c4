/*
 * ebsd_oracle.h -- CPU restatement of CTEMsoft CTEMEBSD's pattern loop.
 * TEST INFRASTRUCTURE ONLY (the checker); PARITY UNPINNED (the reference has
 * no tests or fixtures for this path and cannot be compiled here).
 * See ebsd_oracle.c for the semantics mirrored and the cited source lines.
 */
#ifndef EBSD_ORACLE_H
#define EBSD_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Namelist EBSDdata geometry (CTEMEBSD.f90:112-124) plus the MC tilt sig. */
typedef struct {
    float L, thetac, delta;
    int32_t numsx, numsy;
    float xpc, ypc;
    double sig; /* MC file sample tilt, degrees (CTEMMC.f90:272) */
} oracle_geometry;

/* The same geometry in binary64, for the FP64 re-evaluation and its
 * derivatives (finite differences need steps finer than float spacing). */
typedef struct {
    double L, thetac, delta;
    int32_t numsx, numsy;
    double xpc, ypc;
    double sig;
} oracle_geometry_d;

int oracle_lambert_inverse_f32(const float xyz[3], float res[2]);
int oracle_lambert_inverse_f64(const double xyz[3], double res[2]);
int oracle_lambert_forward_f64(const double xy[2], double res[3]);
void oracle_quat_mult_f32(const float x[4], const float y[4], float r[4]);
void oracle_eu2qu_f32(const float e[3], float res[4]);
void oracle_ax2qu_f32(const float a[4], float res[4]);
void oracle_angles_to_quats_f32(const float* rows, int64_t n, int mode, int hkl,
                                const float axisangle[4], float* quats);

void oracle_detector_f32(const oracle_geometry* g, float* rgx, float* rgy, float* rgz);
void oracle_detector_f64(const oracle_geometry_d* g, double* rgx, double* rgy, double* rgz);

int32_t oracle_mc_weights_f32(const oracle_geometry* g, const float* rgx, const float* rgy,
                              const float* rgz, const int32_t* accum_e, int nE, int nsx,
                              int nsy, int Emin, int Emax, float* W);
double oracle_mc_weights_f64(const oracle_geometry_d* g, const double* rgx, const double* rgy,
                             const double* rgz, const int32_t* accum_e, int nE, int nsx,
                             int nsy, int Emin, int Emax, double* W);
double oracle_prefactor(double beamcurrent, double dwelltime, int32_t num_el);
void oracle_energy_window(float energymin, float energymax, double Ehistmin, double Ebinsize,
                          int numEbins, int* Emin, int* Emax);

float oracle_master_scale_f32(int npx);
void oracle_cells_f32(const oracle_geometry* g, const float* rgx, const float* rgy,
                      const float* rgz, const float* quats, int64_t N, int npx, int npy,
                      int32_t* nix_out, int32_t* niy_out, float* ixy0_out, float* ixy1_out);
void oracle_patterns_f32(const oracle_geometry* g, const float* rgx, const float* rgy,
                         const float* rgz, const float* W, int nE, int Emin, int Emax,
                         const float* sr, int npx, int npy, const float* quats, int64_t N,
                         double prefactor, float* out, int nthreads);
void oracle_patterns_f64(const oracle_geometry_d* g, const double* rgx, const double* rgy,
                         const double* rgz, const double* W, int nE, int Emin, int Emax,
                         const float* sr, int npx, int npy, const double* quats, int64_t N,
                         double prefactor, double* out, int nthreads);

/* Analytic FP64 derivatives (ebsd_oracle_grad.c).  Parameters per pattern:
 * left rotation tangent (w0,w1,w2), q(w) = exp(w) (x) q, and the pattern
 * centre (xpc, ypc, L).  mode 0: cotangent -- grad[n] = sum_B cot[n][B] *
 * dO[n][B]/dphi; mode 1: normalised-dot-product loss against targets
 * (data = targets), loss[n] = 1 - <O,T>/(|O||T|).  O is the output record
 * after prefactor and binning ('lin' for binning > 1). */
void oracle_vjp_f64(const oracle_geometry_d* g, const int32_t* accum_e, int nE, int nsx, int nsy,
                    int Emin, int Emax, const float* sr, int npx, int npy, const double* quats,
                    int64_t N, double prefactor, int binning, int mode, const float* data,
                    double* loss, double* grad, int nthreads);
void oracle_epilogue_f32(const float* pat, int numsx, int numsy, int binning, int mode,
                         float gammavalue, float* out);
void oracle_epilogue_f64(const double* pat, int numsx, int numsy, int binning, int mode,
                         double gammavalue, double* out);
int oracle_max_threads(void);

/* Cubochoric sampling of Rodrigues fundamental zones (ebsd_oracle_so3.c). */
void oracle_so3_constants(double out[8]);
int oracle_cu2ho_d(const double c[3], double res[3]);
int oracle_ho2cu_d(const double h[3], double res[3]);
void oracle_ho2ro_d(const double h[3], double res[3]);
void oracle_cu2ro_d(const double c[3], double rod[3]);
void oracle_ro2qu_d(const double r[3], double q[4]);
int oracle_fz_type(int pgnum, int* order);
int oracle_fz_code(const double rod[3], int type, int order);
int64_t oracle_rfz_axis(int nsteps, double* xs, int64_t cap);
int64_t oracle_sample_rfz(int nsteps, int pgnum, double* rods, int64_t cap);

/* Monte-Carlo backscatter histogram, CTEMMC.f90:307-529 (ebsd_oracle_mc.c).
 * Material numbers are CalcDensity's density [g/cm^3], average Z and
 * average atomic weight [g/mol]. */
typedef struct {
    double sig, omega, EkeV, Ehistmin, Ebinsize, depthmax, depthstep;
    double Ze, density, at_wt;
    int32_t numsx; /* odd number of Lambert points per side */
} oracle_mc_params;
int oracle_mc_dims(const oracle_mc_params* p, int* numEbins, int* numzbins);
int64_t oracle_mc_philox(const oracle_mc_params* p, uint64_t seed, int64_t e0, int64_t e1,
                         int32_t* accum_e, int32_t* accum_z);
int64_t oracle_mc_reference_rng(const oracle_mc_params* p, int32_t primeseed, int nthreads,
                                int64_t num_el, int32_t* accum_e, int32_t* accum_z);
void oracle_mc_uniforms(int kind, uint64_t seed_or_prime, int64_t electron, int count, float* u);
void oracle_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);

#ifdef __cplusplus
}
#endif
#endif
