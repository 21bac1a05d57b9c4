// Internal declarations shared by the translation units of libebsdgpu.so.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "../../include/ebsd_gpu.h"

namespace ebsd {

// Largest energy window the kernels are instantiated for: NV float4 vectors
// of bins per master node (NV = ceil(nEsel/4)).
constexpr int kMaxNV = 16;

// Launch shapes the forward kernels accept.
constexpr int kTileX = 32;  // pixels along x per CTA

struct DeviceBuf {
    void* ptr = nullptr;
    size_t bytes = 0;
};

// Everything a forward-type kernel needs; filled by the C-ABI layer.
struct FwdParams {
    const float4* master;  // [gy][gx][NV] float4, bins Emin..Emax, zero padded
    const float4* rg;      // [P] detector direction cosines (x, y, z, 0)
    const float4* W;       // [NV][P] energy weights (float4 planes)
    const float4* quats;   // [n] scalar-first quaternions
    float* out;            // [n][out_ny][out_nx]
    int64_t n;
    int numsx, numsy, P;
    int npx, npy, gx;      // gx: the interleaved master's row pitch in nodes
    float scl, spi2;       // sngl(npx/sPio2), sngl(sPi2)
    double prefactor;
    int binning, mode;     // EBSD_SCALING_*
    float gammavalue, bindx;
    int out_nx, out_ny;
    int poisson;
    int gamma_fast;        // 'gam' with a positive, finite, non-integer exponent (see gamma_pow)
    uint64_t seed;
    int64_t o_offset;      // index of quats[0] within the call (noise streams)
    int accurate;          // 1: cancellation-free 1 - z near the poles; 2: binary64 geometry
    const double* rg64;    // [3][P] binary64 directions (accurate == 2)
    double scl64;          // npx / sqrt(pi/2) in binary64
    // diagnostics (the cells instantiation of the pattern kernel): [n][P]
    int32_t* nix;
    int32_t* niy;
    float* ixy0;
    float* ixy1;
};

// Adjoint-only inputs and outputs (ebsd_vjp.cu).  Pointers are offset to
// the current chunk of orientations by the caller.
struct VjpParams {
    const float4* drg;   // [3][P] d rg / d(xpc, ypc, L)
    const float4* dW;    // [2NV+1][P]: dW/d(xpc, ypc, L) = G0 di0 + G1 di1; planes
                         // 0..NV-1 G0, NV..2NV-1 G1, 2NV di1 (di0 in drg's .w)
    const float* data;   // [n][out_ny][out_nx] cotangent or targets
    float* partial;      // scratch [n][ntiles][K]
    float* loss;         // [n] or null
    float* grad;         // [n][6]
    int binning;         // 1 for 'not'
    int opc;             // orientations per CTA
};

// Batched pattern loop (ebsd_forward.cu).  A queued job runs at its
// handle's tile height (32 x 4, 8 or 16 pixels, raised until binned records
// hold whole blocks); 8x8-binned jobs (BIN8) take 8 or 16 rows.
inline bool batch_shape_ok(int ty, bool bin8)
{
    return (ty == 4 && !bin8) || ty == 8 || ty == 16;
}

struct BatchJob {
    FwdParams p;            // detector, master, quats, out, epilogue of the job
    int tiles_x, ntiles, opc, pad;
    long long item_begin;   // first work item of this job in the queue
    long long items;        // ntiles * ceil(n / opc)
};

// One launch of the persistent queue kernel: its jobs travel in the kernel's
// parameters (the constant bank, read through the constant cache; a kernel
// takes up to 32 764 bytes of parameters), at most kBatchLaunchJobs of them.
constexpr int kBatchLaunchJobs = 128;
struct BatchLaunch {
    long long total_items;  // items of all jobs, in job order
    int njobs, pad;
    BatchJob job[kBatchLaunchJobs];
};
static_assert(sizeof(BatchLaunch) + 8 <= 32764, "kernel parameters above the 32 KB limit");

// Launch configuration picked by the tuner or by default.
struct LaunchCfg {
    int tile_y = 4;        // CTA is 32 x tile_y pixels (raised to 8 for binning 8)
    int orient_per_cta = 0;  // 0: chosen per launch from the grid size
    int warp_w = 16;         // pixels along x per warp: 16 (16 x 2) or 32 (32 x 1)
    bool strict = false;   // reference summation order in the gather
    // L2 access-policy window kept persisting for the master pattern
    const void* persist_base = nullptr;
    size_t persist_bytes = 0;
    float persist_hit_ratio = 0.0f;
};

// Attach the master's persisting-L2 window to a launch (no-op when unset).
inline void set_persist_attr(const LaunchCfg& cfg, cudaLaunchAttribute* attr,
                             cudaLaunchConfig_t& lc)
{
    lc.attrs = attr;
    lc.numAttrs = 0;
    if (!cfg.persist_base || cfg.persist_bytes == 0) return;
    attr[0].id = cudaLaunchAttributeAccessPolicyWindow;
    attr[0].val.accessPolicyWindow.base_ptr = const_cast<void*>(cfg.persist_base);
    attr[0].val.accessPolicyWindow.num_bytes = cfg.persist_bytes;
    attr[0].val.accessPolicyWindow.hitRatio = cfg.persist_hit_ratio;
    attr[0].val.accessPolicyWindow.hitProp = cudaAccessPropertyPersisting;
    attr[0].val.accessPolicyWindow.missProp = cudaAccessPropertyStreaming;
    lc.numAttrs = 1;
}

// Row pitch (in nodes) of the energy-interleaved master: 2 npx + 1 nodes,
// padded to the next pitch with NV * pitch = 4 (mod 8) float4 (NV not a
// multiple of 8).  A warp's 128-bit loads that hit L1 are served 8 lanes at
// a time from the banked data array, 16 bytes per bank group (8 groups),
// and two different 16-byte chunks in one group cost a second wavefront,
// whichever lines they come from.  With that pitch the group of node
// (x + dx, y + dy) differs from node (x, y)'s for every |dx| <= 2, |dy| <= 1
// (NV = 3: 3 dx + 4 dy != 0 mod 8); at 2 npx + 1 = 1001 the anti-diagonal
// neighbour shared the node's groups.  Measured at 640x480, 10 000
// orientations: 285.0 k patterns/s unpadded, 292.8 k padded (1004 nodes).
inline int master_pitch(int npx, int NV)
{
    int pitch = 2 * npx + 1;
    if (NV % 8 != 0)
        while ((NV * pitch) % 8 != 4) ++pitch;
    return pitch;
}

// Setup-stage kernels (ebsd_setup.cu).
cudaError_t launch_master_relayout(const float* raw, int npx, int npy, int nE, int numset,
                                   int e0, int nsel, int NV, float4* il, cudaStream_t s);
cudaError_t launch_detector(const ebsd_geometry& g, float ca, float sa, float4* rg,
                            cudaStream_t s);
// binary64 directions, [3][P] (x, y, z planes)
cudaError_t launch_detector64(const ebsd_geometry& g, double* rg64, cudaStream_t s);
cudaError_t launch_weights(const float4* rg, int P, const int32_t* accum_e, int nE, int nsx,
                           int nsy, float sclmc, float spi2, int e0, int nsel, int NV, int fp64,
                           const ebsd_geometry& g, float4* W, float4* Wref, cudaStream_t s);
cudaError_t launch_num_el(const float4* W, int P, int nsel, int NV, float* sum_out,
                          cudaStream_t s);

cudaError_t launch_geom_derivs(const ebsd_geometry& g, const int32_t* accum_e, int nE, int nsx,
                               int nsy, int e0, int nsel, int NV, float4* drg, float4* dW,
                               cudaStream_t s);

// Adjoint (ebsd_vjp.cu).
int vjp_tiles(const FwdParams& p, int tile_y);
cudaError_t launch_vjp(const FwdParams& p, const VjpParams& vp, int NV, int mode, int tile_y,
                       cudaStream_t s);

// Gauss-Newton (ebsd_vjp.cu): sys holds 28 doubles per pattern.
constexpr int kGnPartialK = 36;
constexpr int kGnSysK = 28;
cudaError_t launch_gn_accumulate(const FwdParams& p, const VjpParams& vp, int NV, int tile_y,
                                 double* sys, float* loss, cudaStream_t s);
int gn_schur_blocks(int64_t n);
cudaError_t launch_gn_schur(const double* sys, int64_t n, double lambda, double* partial,
                            double* out, cudaStream_t s);
cudaError_t launch_gn_update(const double* sys, int64_t n, double lambda, const double* dpc,
                             float4* quats, float* step, cudaStream_t s);

// Memory-hierarchy read bandwidth (ebsd_membw.cu), level EBSD_BW_*.
cudaError_t measure_read_bandwidth(int device, int level, long long bytes, int repeats,
                                   double* gbs, double* seconds);

// Pattern kernels (ebsd_forward.cu).
// CTAs that launch_forward would start for p under cfg.
int64_t forward_ctas(const FwdParams& p, const LaunchCfg& cfg);
// cells: the diagnostic instantiation that also stores p.nix/niy/ixy0/ixy1.
cudaError_t launch_forward(const FwdParams& p, int NV, const LaunchCfg& cfg, cudaStream_t s,
                           bool cells = false);
cudaError_t launch_forward_batched(const BatchLaunch& L, unsigned long long* counter, int NV,
                                   bool noise, int ty, bool bin8, int grid, cudaStream_t s);
int batched_grid(int NV, bool noise, int ty, bool bin8);

// Cubochoric fundamental-zone sampling (ebsd_so3.cu).  Constants of
// Lambert.f90:246-280 in binary64.
struct So3Consts {
    double Pi, sPi, srt, pref, semi, sc, R1, r2, r22, pi12, pi8, prek, r24, rvmax2, edge;
    double BP[6];
};
So3Consts so3_constants();
constexpr int kMaxRfzSteps = 1000;  // (2N+1)^3 codes: 8 GB at the limit
long long rfz_chunks(long long total);
size_t rfz_chunk_bytes();
// code: m^3 bytes; chunk: rfz_chunks * rfz_chunk_bytes; enter/offset: one
// per chunk; count: one value.  rods (3 doubles) / quats (float4) may be
// null; at most cap entries are written.
cudaError_t launch_rfz(const So3Consts& K, const double* xs, int m, int type, int order,
                       uint8_t* code, void* chunk, int* enter, long long* offset,
                       long long* count, long long cap, double* rods, float* quats,
                       bool count_only, cudaStream_t s);

// Monte-Carlo backscatter histograms (ebsd_mc.cu): CTEMMC.f90:410-440
// derived constants.
struct McConsts {
    double EkeV, Ehistmin, Ebinsize, depthstep, Ze, Emin, pre, prealpha, J, predEds, tpi, tano,
        delta, sPi2, cxstart, czstart;
    int nx, nz10, numEbins, numzbins;
};
McConsts mc_constants(const ebsd_mc_params& p);
cudaError_t launch_mc(const McConsts& K, uint64_t seed, long long e0, long long n,
                      int32_t* accum_e, int32_t* accum_z, unsigned long long* counted,
                      bool fp32, cudaStream_t s);

}  // namespace ebsd
