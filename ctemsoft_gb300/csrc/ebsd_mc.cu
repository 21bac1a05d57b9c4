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

__device__ __forceinline__ void free_path(const McConsts& K, double Ec, double& alpha,
                                          double& lambda)
{
    alpha = K.prealpha / Ec;
    const double step = Ec * (Ec + 1024.0) / K.Ze / (Ec + 511.0);
    const double sige = kPresig * step * step * alpha * (1.0 + alpha);
    lambda = K.pre * sige;
}

// Record an exit (CTEMMC.f90:487-515); returns 1 if counted in accum_e.
__device__ int record_exit(const McConsts& K, double Ec, const double xyz[3], const double cp[3],
                           int32_t* __restrict__ accum_e, int32_t* __restrict__ accum_z)
{
    // Lambert.f90:452-483, binary64 square-Lambert inverse, scaled
    double X = 0.0, Y = 0.0;
    const double n = cp[0] * cp[0] + cp[1] * cp[1] + cp[2] * cp[2];
    if (!(fabs(1.0 - n) > 1.0e-12) && fabs(cp[2]) != 1.0) {
        if (fabs(cp[1]) <= fabs(cp[0])) {
            const double q = fabs(cp[0]) / cp[0] * sqrt(2.0 * (1.0 - cp[2]));
            X = q * K.sPi2;
            Y = q * atan(cp[1] / cp[0]) / K.sPi2;
        } else {
            const double q = fabs(cp[1]) / cp[1] * sqrt(2.0 * (1.0 - cp[2]));
            X = q * atan(cp[0] / cp[1]) / K.sPi2;
            Y = q * K.sPi2;
        }
    }
    X = K.delta * X;
    Y = K.delta * Y;
    // a NaN direction passes the norm test above (as in the reference);
    // rounding it would give an arbitrary index, so it is not counted
    if (!isfinite(X) || !isfinite(Y)) return 0;
    // nearest pixel with the frame reversal (x, y) -> (y, -x); nint = round half away
    const long long ix = llround(Y), iy = llround(-X);
    if (llabs(ix) > K.nx || llabs(iy) > K.nx || !(Ec > K.Emin)) return 0;
    const long long iE = llround((Ec - K.Ehistmin) / K.Ebinsize) + 1;
    if (iE < 1 || iE > K.numEbins) return 0;  // the reference does not check
    const double edis = fabs(xyz[2] / cp[2]);
    const double zb = edis * 0.1 / K.depthstep;
    const long long iz = zb < 1.0e15 ? llround(zb) + 1 : -1;  // inf/NaN: no depth bin
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

__global__ void __launch_bounds__(256) k_mc(const McConsts K, uint64_t seed, long long e0,
                                            long long n, int32_t* __restrict__ accum_e,
                                            int32_t* __restrict__ accum_z,
                                            unsigned long long* __restrict__ counted)
{
    const long long stride = (long long)gridDim.x * blockDim.x;
    long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    unsigned long long mine = 0;
    Stream rng;
    double Ec = 0.0, alpha = 0.0, lambda = 0.0, step = 0.0;
    double xyz[3], cxyz[3];
    int traj = kMaxSteps;  // "no electron in flight"
    for (;;) {
        if (traj >= kMaxSteps) {  // start the next electron (CTEMMC.f90:444-466)
            if (k >= n) break;
            rng.start(seed, e0 + k);
            k += stride;
            Ec = K.EkeV;
            free_path(K, Ec, alpha, lambda);
            step = -lambda * log(rng.next());
            cxyz[0] = K.cxstart;
            cxyz[1] = 0.0;
            cxyz[2] = K.czstart;
            for (int i = 0; i < 3; ++i) xyz[i] = 0.0 + step * kScaled * cxyz[i];
            traj = 0;
        }
        // one scattering step (CTEMMC.f90:469-521)
        const double dEds = K.predEds * log(Ec * K.J + 1.0) / Ec;
        Ec = Ec + dEds * step;
        if (Ec < kMinEnergy) {
            traj = kMaxSteps;
            continue;
        }
        const double r1 = rng.next();
        const double cphi = 1.0 - 2.0 * alpha * r1 / (1.0 + alpha - r1);
        const double sphi = sin(acos(cphi));
        const double psi = K.tpi * rng.next();
        double spsi, cpsi;
        sincos(psi, &spsi, &cpsi);
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
        free_path(K, Ec, alpha, lambda);
        step = -lambda * log(rng.next());
        double xn[3];
        for (int i = 0; i < 3; ++i) xn[i] = xyz[i] + step * kScaled * cp[i];
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

int mc_grid()
{
    int dev = 0, sms = 0, per = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_mc, 256, 0);
    return sms * (per > 0 ? per : 1);
}

cudaError_t launch_mc(const McConsts& K, uint64_t seed, long long e0, long long n,
                      int32_t* accum_e, int32_t* accum_z, unsigned long long* counted,
                      cudaStream_t s)
{
    if (n <= 0) return cudaSuccess;
    const long long want = (n + 255) / 256;
    const int grid = (int)std::min<long long>(want, (long long)mc_grid());
    k_mc<<<grid, 256, 0, s>>>(K, seed, e0, n, accum_e, accum_z, counted);
    return cudaGetLastError();
}

}  // namespace ebsd
