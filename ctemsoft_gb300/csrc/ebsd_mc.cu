// Monte-Carlo backscatter histogram of CTEMMC (CTEMMC.f90:307-529, CSDA
// mode): electrons enter a tilted sample, lose energy continuously (Joy-Luo
// stopping power), scatter elastically (screened Rutherford), and those that
// leave through the surface are counted on the modified square-Lambert grid
// of exit directions by exit energy (accum_e) and, coarser, by exit depth
// (accum_z).  Arithmetic is binary64 as in the reference.
//
// Random numbers: the reference runs a few long sequential streams, which a
// GPU cannot reproduce draw for draw (how many numbers an electron consumes
// depends on its path).  Each electron here has its own Philox4x32-10
// stream -- key = seed, counter = (block, 0, electron index) -- and a
// 32-bit word w becomes the reference's single-precision uniform
// real(0.5d0 + 0.23283064d-9*w) (rng.f95), so results depend only on the
// seed and the electron range, not on the launch shape or the GPU count.
//
// One thread runs one electron at a time in a single flattened loop: a lane
// whose electron finishes starts its next one on the next iteration, so a
// warp stays inside the step body instead of waiting for its longest
// trajectory.  Counts are added with integer atomics.
#include <algorithm>
#include <cmath>
#include <cstdint>

#include "ebsd_internal.h"
#include "ebsd_noise.cuh"

namespace ebsd {

namespace {

constexpr double kPresig = 1.5273987e19, kScaled = 1.0e8, kMinEnergy = 1.0;
constexpr int kMaxSteps = 5000;  // CTEMMC.f90:431

struct Stream {
    uint32_t k0, k1, e_lo, e_hi, block;
    uint32_t b0, b1, b2, b3;
    int pos;
    __device__ void start(uint64_t seed, long long e)
    {
        k0 = (uint32_t)seed;
        k1 = (uint32_t)(seed >> 32);
        e_lo = (uint32_t)e;
        e_hi = (uint32_t)((unsigned long long)e >> 32);
        block = 0;
        pos = 4;
    }
    __device__ double next()
    {
        if (pos == 4) {
            const Philox4 r = philox4x32_10(block, 0u, e_lo, e_hi, k0, k1);
            b0 = r.v[0];
            b1 = r.v[1];
            b2 = r.v[2];
            b3 = r.v[3];
            pos = 0;
            ++block;
        }
        const uint32_t w = pos == 0 ? b0 : pos == 1 ? b1 : pos == 2 ? b2 : b3;
        ++pos;
        // rng.f95: u = real(0.5d0 + 0.23283064d-9 * imz), a single-precision value
        return (double)(float)(0.5 + 0.23283064e-9 * (double)(int32_t)w);
    }
};

// Arithmetic of one precision: binary64 (the reference's, the default) or
// binary32 (option mc_fp32: the same steps in single precision; the float
// Lambert inverse takes the single-precision norm tolerance of
// Lambert.f90:405-436).
template <typename T>
struct Math;
template <>
struct Math<double> {
    static constexpr double kNormEps = 1.0e-12;
    __device__ static double log_(double x) { return log(x); }
    __device__ static double sin_(double x) { return sin(x); }
    __device__ static double acos_(double x) { return acos(x); }
    __device__ static double sqrt_(double x) { return sqrt(x); }
    __device__ static double atan_(double x) { return atan(x); }
    __device__ static void sincos_(double x, double* s, double* c) { sincos(x, s, c); }
    __device__ static long long round_(double x) { return llround(x); }
};
template <>
struct Math<float> {
    static constexpr float kNormEps = 1.0e-6f;
    __device__ static float log_(float x) { return logf(x); }
    __device__ static float sin_(float x) { return sinf(x); }
    __device__ static float acos_(float x) { return acosf(x); }
    __device__ static float sqrt_(float x) { return sqrtf(x); }
    __device__ static float atan_(float x) { return atanf(x); }
    __device__ static void sincos_(float x, float* s, float* c) { sincosf(x, s, c); }
    __device__ static long long round_(float x) { return llroundf(x); }
};

// McConsts in the working precision.
template <typename T>
struct Kc {
    T EkeV, Ehistmin, Ebinsize, depthstep, Ze, Emin, pre, prealpha, J, predEds, tpi, tano, delta,
        sPi2, cxstart, czstart, presig, scaled, min_energy;
    int nx, nz10, numEbins, numzbins;
    __device__ explicit Kc(const McConsts& K)
        : EkeV((T)K.EkeV), Ehistmin((T)K.Ehistmin), Ebinsize((T)K.Ebinsize),
          depthstep((T)K.depthstep), Ze((T)K.Ze), Emin((T)K.Emin), pre((T)K.pre),
          prealpha((T)K.prealpha), J((T)K.J), predEds((T)K.predEds), tpi((T)K.tpi),
          tano((T)K.tano), delta((T)K.delta), sPi2((T)K.sPi2), cxstart((T)K.cxstart),
          czstart((T)K.czstart), presig((T)kPresig), scaled((T)kScaled),
          min_energy((T)kMinEnergy), nx(K.nx), nz10(K.nz10), numEbins(K.numEbins),
          numzbins(K.numzbins)
    {
    }
};

template <typename T>
__device__ __forceinline__ void free_path(const Kc<T>& K, T Ec, T& alpha, T& lambda)
{
    alpha = K.prealpha / Ec;
    const T step = Ec * (Ec + (T)1024.0) / K.Ze / (Ec + (T)511.0);
    const T sige = K.presig * step * step * alpha * ((T)1.0 + alpha);
    lambda = K.pre * sige;
}

// Record an exit (CTEMMC.f90:487-515); returns 1 if counted in accum_e.
template <typename T>
__device__ int record_exit(const Kc<T>& K, T Ec, const T xyz[3], const T cp[3],
                           int32_t* __restrict__ accum_e, int32_t* __restrict__ accum_z)
{
    using F = Math<T>;
    // Lambert.f90:452-483 (binary64) / :405-436 (binary32) square-Lambert
    // inverse, scaled
    T X = 0, Y = 0;
    const T n = cp[0] * cp[0] + cp[1] * cp[1] + cp[2] * cp[2];
    if (!(fabs((T)1.0 - n) > F::kNormEps) && fabs(cp[2]) != (T)1.0) {
        if (fabs(cp[1]) <= fabs(cp[0])) {
            const T q = fabs(cp[0]) / cp[0] * F::sqrt_((T)2.0 * ((T)1.0 - cp[2]));
            X = q * K.sPi2;
            Y = q * F::atan_(cp[1] / cp[0]) / K.sPi2;
        } else {
            const T q = fabs(cp[1]) / cp[1] * F::sqrt_((T)2.0 * ((T)1.0 - cp[2]));
            X = q * F::atan_(cp[0] / cp[1]) / K.sPi2;
            Y = q * K.sPi2;
        }
    }
    X = K.delta * X;
    Y = K.delta * Y;
    // a NaN direction passes the norm test above (as in the reference);
    // rounding it would give an arbitrary index, so it is not counted
    if (!isfinite(X) || !isfinite(Y)) return 0;
    // nearest pixel with the frame reversal (x, y) -> (y, -x); nint = round half away
    const long long ix = F::round_(Y), iy = F::round_(-X);
    if (llabs(ix) > K.nx || llabs(iy) > K.nx || !(Ec > K.Emin)) return 0;
    const long long iE = F::round_((Ec - K.Ehistmin) / K.Ebinsize) + 1;
    if (iE < 1 || iE > K.numEbins) return 0;  // the reference does not check
    const T edis = fabs(xyz[2] / cp[2]);
    const T zb = edis * (T)0.1 / K.depthstep;
    const long long iz = zb < (T)1.0e15 ? F::round_(zb) + 1 : -1;  // inf/NaN: no depth bin
    if (iz > 0 && iz <= K.numzbins && accum_z) {
        const long long px = llroundf((float)ix / 10.0f), py = llroundf((float)iy / 10.0f);
        if (llabs(px) <= K.nz10 && llabs(py) <= K.nz10) {
            const long long w = 2 * K.nz10 + 1;
            atomicAdd(accum_z + (iE - 1) +
                          (long long)K.numEbins *
                              ((iz - 1) + (long long)K.numzbins * ((px + K.nz10) + w * (py + K.nz10))),
                      1);
        }
    }
    const long long g = 2 * K.nx + 1;
    atomicAdd(accum_e + (iE - 1) + (long long)K.numEbins * ((ix + K.nx) + g * (iy + K.nx)), 1);
    return 1;
}

template <typename T>
__global__ void __launch_bounds__(256, 4) k_mc(const McConsts KD, uint64_t seed, long long e0,
                                            long long n, int32_t* __restrict__ accum_e,
                                            int32_t* __restrict__ accum_z,
                                            unsigned long long* __restrict__ counted)
{
    using F = Math<T>;
    const Kc<T> K(KD);
    const long long stride = (long long)gridDim.x * blockDim.x;
    long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    unsigned long long mine = 0;
    Stream rng;
    T Ec = 0, alpha = 0, lambda = 0, step = 0;
    T xyz[3], cxyz[3];
    int traj = kMaxSteps;  // "no electron in flight"
    for (;;) {
        if (traj >= kMaxSteps) {  // start the next electron (CTEMMC.f90:444-466)
            if (k >= n) break;
            rng.start(seed, e0 + k);
            k += stride;
            Ec = K.EkeV;
            free_path(K, Ec, alpha, lambda);
            step = -lambda * F::log_((T)rng.next());
            cxyz[0] = K.cxstart;
            cxyz[1] = 0;
            cxyz[2] = K.czstart;
            for (int i = 0; i < 3; ++i) xyz[i] = (T)0.0 + step * K.scaled * cxyz[i];
            traj = 0;
        }
        // one scattering step (CTEMMC.f90:469-521)
        const T dEds = K.predEds * F::log_(Ec * K.J + (T)1.0) / Ec;
        Ec = Ec + dEds * step;
        if (Ec < K.min_energy) {
            traj = kMaxSteps;
            continue;
        }
        const T r1 = (T)rng.next();
        const T cphi = (T)1.0 - (T)2.0 * alpha * r1 / ((T)1.0 + alpha - r1);
        const T sphi = F::sin_(F::acos_(cphi));
        const T psi = K.tpi * (T)rng.next();
        T spsi, cpsi;
        F::sincos_(psi, &spsi, &cpsi);
        T cp[3];
        if (fabs(cxyz[2]) > (T)0.99999) {
            cp[0] = sphi * cpsi;
            cp[1] = sphi * spsi;
            cp[2] = (cxyz[2] / fabs(cxyz[2])) * cphi;
        } else {
            const T dsq = F::sqrt_((T)1.0 - cxyz[2] * cxyz[2]);
            const T dsqi = (T)1.0 / dsq;
            cp[0] = sphi * (cxyz[0] * cxyz[2] * cpsi - cxyz[1] * spsi) * dsqi + cxyz[0] * cphi;
            cp[1] = sphi * (cxyz[1] * cxyz[2] * cpsi + cxyz[0] * spsi) * dsqi + cxyz[1] * cphi;
            cp[2] = -(sphi * cpsi * dsq) + cxyz[2] * cphi;
        }
        const T dd = (T)1.0 / F::sqrt_(cp[0] * cp[0] + cp[1] * cp[1] + cp[2] * cp[2]);
        for (int i = 0; i < 3; ++i) cp[i] = cp[i] * dd;
        free_path(K, Ec, alpha, lambda);
        step = -lambda * F::log_((T)rng.next());
        T xn[3];
        for (int i = 0; i < 3; ++i) xn[i] = xyz[i] + step * K.scaled * cp[i];
        if (xn[2] > xn[1] * K.tano) {  // left the (double-tilted) surface
            mine += (unsigned long long)record_exit(K, Ec, xyz, cp, accum_e, accum_z);
            traj = kMaxSteps;
            continue;
        }
        for (int i = 0; i < 3; ++i) {
            cxyz[i] = cp[i];
            xyz[i] = xn[i];
        }
        ++traj;
    }
    for (int off = 16; off > 0; off >>= 1) mine += __shfl_xor_sync(0xffffffffu, mine, off);
    if ((threadIdx.x & 31) == 0 && mine) atomicAdd(counted, mine);
}

}  // namespace

// CTEMMC.f90:410-440, and LPs%sPio2 / LPs%sPi2 (Lambert.f90:252-253).  The
// reference's own constants: truncated pi and degree factor, single-precision
// literals 0.67 and 1.166.
McConsts mc_constants(const ebsd_mc_params& p)
{
    const double kPi = 3.141592653589, kAvogadro = 6.0221415e+23, kDtoR = 0.017453293;
    McConsts K;
    K.EkeV = p.EkeV;
    K.Ehistmin = p.Ehistmin;
    K.Ebinsize = p.Ebinsize;
    K.depthstep = p.depthstep;
    K.Ze = p.Ze;
    K.numEbins = (int)((p.EkeV - p.Ehistmin) / p.Ebinsize) + 1;
    K.numzbins = (int)(p.depthmax / p.depthstep) + 1;
    K.nx = (p.numsx - 1) / 2;
    K.nz10 = K.nx / 10;
    K.Emin = p.Ehistmin - p.Ebinsize / 2.0;
    K.pre = p.at_wt / kAvogadro / p.density;
    K.prealpha = 3.4e-3 * std::pow(p.Ze, (double)0.67f);
    const double J = (9.76 * p.Ze + 58.5 / std::pow(p.Ze, 0.19)) * 1.0e-3 / (double)1.166f;
    K.J = 1.0 / J;
    K.predEds = -78500.0 * p.density * p.Ze / p.at_wt;
    K.tpi = 2.0 * kPi;
    K.tano = std::tan(p.omega * kDtoR);
    const double dpi = 4.0 * std::atan(1.0);
    K.delta = (double)K.nx / std::sqrt(dpi * 0.5);
    K.sPi2 = std::sqrt(dpi) * 0.5;
    K.cxstart = std::cos((90.0 - p.sig) * kDtoR);
    K.czstart = -std::sin((90.0 - p.sig) * kDtoR);
    return K;
}

template <typename T>
int mc_grid()
{
    int dev = 0, sms = 0, per = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_mc<T>, 256, 0);
    return sms * (per > 0 ? per : 1);
}

cudaError_t launch_mc(const McConsts& K, uint64_t seed, long long e0, long long n,
                      int32_t* accum_e, int32_t* accum_z, unsigned long long* counted,
                      bool fp32, cudaStream_t s)
{
    if (n <= 0) return cudaSuccess;
    const long long want = (n + 255) / 256;
    if (fp32) {
        const int grid = (int)std::min<long long>(want, (long long)mc_grid<float>());
        k_mc<float><<<grid, 256, 0, s>>>(K, seed, e0, n, accum_e, accum_z, counted);
    } else {
        const int grid = (int)std::min<long long>(want, (long long)mc_grid<double>());
        k_mc<double><<<grid, 256, 0, s>>>(K, seed, e0, n, accum_e, accum_z, counted);
    }
    return cudaGetLastError();
}

}  // namespace ebsd
