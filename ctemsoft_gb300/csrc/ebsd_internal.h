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
constexpr int kTileX = 32;  // pixels along x per CTA row (one warp)

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
    int npx, npy, gx;
    float scl, spi2;       // sngl(npx/sPio2), sngl(sPi2)
    double prefactor;
    int binning, mode;     // EBSD_SCALING_*
    float gammavalue, bindx;
    int out_nx, out_ny;
    int poisson;
    uint64_t seed;
    int accurate;          // cancellation-free 1 - z near the poles
    // diagnostics (cells mode)
    int32_t* nix;
    int32_t* niy;
    float* ixy0;
    float* ixy1;
};

// Launch configuration picked by the tuner or by default.
struct LaunchCfg {
    int tile_y = 8;        // CTA is 32 x tile_y pixels
    int orient_per_cta = 4;
};

// Setup-stage kernels (ebsd_setup.cu).
cudaError_t launch_master_relayout(const float* raw, int npx, int npy, int nE, int numset,
                                   int e0, int nsel, int NV, float4* il, cudaStream_t s);
cudaError_t launch_detector(const ebsd_geometry& g, float ca, float sa, float4* rg,
                            cudaStream_t s);
cudaError_t launch_weights(const float4* rg, int P, const int32_t* accum_e, int nE, int nsx,
                           int nsy, float sclmc, float spi2, int e0, int nsel, int NV, int fp64,
                           const ebsd_geometry& g, float4* W, float4* Wref, cudaStream_t s);
cudaError_t launch_num_el(const float4* W, int P, int nsel, int NV, float* sum_out,
                          cudaStream_t s);

// Pattern kernels (ebsd_forward.cu).
cudaError_t launch_forward(const FwdParams& p, int NV, const LaunchCfg& cfg, cudaStream_t s);
cudaError_t launch_cells(const FwdParams& p, int NV, cudaStream_t s);

}  // namespace ebsd
