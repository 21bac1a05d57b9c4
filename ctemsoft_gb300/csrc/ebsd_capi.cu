// C ABI of libebsdgpu.so: handle life cycle, set-up stages and the pattern
// loop with host or device buffers.  See include/ebsd_gpu.h.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <initializer_list>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <utility>
#include <vector>

#include "ebsd_host.h"
#include "ebsd_internal.h"

using namespace ebsd;

// A master pattern on one device, shared by every handle that uses it
// (ebsd_share_master): the raw Fortran-order upload and one
// energy-interleaved layout per energy window (first bin, bin count).
struct MasterStore {
    int device = 0;
    float* raw = nullptr;
    int npx = 0, npy = 0, nE = 0, numset = 0;
    float max_sr = 0.0f;
    std::map<std::pair<int, int>, std::pair<float4*, size_t>> layouts;
    ~MasterStore()
    {
        cudaSetDevice(device);
        cudaFree(raw);
        for (auto& kv : layouts) cudaFree(kv.second.first);
        cudaGetLastError();
    }
};

// Detector tables on one device (direction cosines, weights, derivative
// tables), shared by every handle that took them with ebsd_share_detector.
// A handle that changes its geometry while others hold the same tables gets
// tables of its own first (copy on write), so a sharing handle never sees
// another's geometry.
struct DetectorTables {
    int device = 0;
    float4* rg = nullptr;
    float4* W = nullptr;
    float4* drg = nullptr;
    float4* dW = nullptr;
    double* rg64 = nullptr;  // [3][P] binary64 directions (binary64-geometry mode)
    int P = 0, NV = 0;
    ~DetectorTables()
    {
        cudaSetDevice(device);
        cudaFree(rg64);
        cudaFree(rg);
        cudaFree(W);
        cudaFree(drg);
        cudaFree(dW);
        cudaGetLastError();
    }
};

// An MC energy histogram uploaded to one device; read-only once uploaded,
// so handles share it freely.
struct HistogramStore {
    int device = 0;
    int32_t* ptr = nullptr;
    size_t bytes = 0;
    ~HistogramStore()
    {
        cudaSetDevice(device);
        cudaFree(ptr);
        cudaGetLastError();
    }
};

struct ebsd_handle {
    int device = 0;
    cudaStream_t own_stream = nullptr;
    cudaStream_t stream = nullptr;   // where work is issued
    cudaStream_t copy_stream = nullptr;
    std::string err;

    // master pattern (possibly shared with other handles on this device)
    std::shared_ptr<MasterStore> ms;
    int npx = 0, npy = 0, nE = 0, numset = 0;
    bool have_master = false;

    // energy-interleaved master for the detector's window (owned by ms)
    float4* d_master_il = nullptr;
    size_t il_bytes = 0;

    // detector
    bool have_detector = false;
    ebsd_geometry geom{};
    int Emin = 0, Emax = 0, nsel = 0, NV = 0;
    int32_t num_el = 0;
    std::shared_ptr<DetectorTables> det;  // owner of the four tables below
    float4* d_rg = nullptr;
    float4* d_W = nullptr;
    float4* d_drg = nullptr;   // [3][P] d rg / d(xpc, ypc, L)
    float4* d_dW = nullptr;    // [2NV+1][P] factors of d W / d(xpc, ypc, L) (see VjpParams)
    int P = 0;
    int nsx = 0, nsy = 0;

    // per-call buffers
    DeviceBuf quats[2];
    DeviceBuf outb[2];
    DeviceBuf tmp;
    std::shared_ptr<HistogramStore> accum;  // MC histogram, kept for geometry updates
    DeviceBuf small;           // set-up scalars (num_el sum)
    DeviceBuf wref;            // the reference's single-precision weights (num_el)
    DeviceBuf vjp_partial;     // per-CTA partial sums of the adjoint
    DeviceBuf gn_sys;          // per-pattern Gauss-Newton systems (28 doubles)
    DeviceBuf gn_aux;          // Schur partials, centre system, centre step, steps
    int64_t gn_n = 0;
    DeviceBuf vjp_io;          // device copies of host quats / data / outputs
    float* pinned[2] = {nullptr, nullptr};
    size_t pinned_bytes = 0;
    cudaEvent_t ev_comp[2] = {nullptr, nullptr};
    cudaEvent_t ev_d2h[2] = {nullptr, nullptr};

    // L2 persistence
    int max_persist = 0, max_window = 0;

    LaunchCfg cfg;
    int mc_fp32 = 0;     // Monte-Carlo trajectories in binary32
    int host_direct = 1; // kernel stores straight into pinned host outputs
    int vjp_tile_y = 0;  // adjoint / Gauss-Newton tile height; 0: the defaults below
    int vjp_opc = 0;     // adjoint orientations per CTA; 0: 16 unbinned, 8 binned
    int gn_opc = 32;     // Gauss-Newton orientations per CTA
    int weights_fp64 = 1;
    int lambert_accurate = 0;
    int64_t noise_offset = 0;  // pattern index of a call's first orientation (noise streams)

    // batched pattern loop: device job table, pinned host mirror, graph
    DeviceBuf batch_table;     // the queue counters of the batch's launches
    cudaGraphExec_t batch_exec = nullptr;
    std::vector<int> batch_key;
    cudaStream_t batch_stream = nullptr;
    std::map<int, int> batch_grid;  // NV -> persistent grid size

    // fundamental-zone sampler: codes, chunk scan, device copies of outputs
    DeviceBuf rfz;
    DeviceBuf rfz_out;
    // Monte-Carlo histograms staged for host outputs, and the counter
    DeviceBuf mc;
};

namespace {

thread_local std::string g_err;

int set_err(ebsd_handle* h, int code, const char* fmt, ...)
{
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    if (h)
        h->err = buf;
    else
        g_err = buf;
    return code;
}

int cuda_err(ebsd_handle* h, cudaError_t e, const char* what)
{
    return set_err(h, e == cudaErrorMemoryAllocation ? EBSD_ENOMEM : EBSD_ECUDA, "%s: %s", what,
                   cudaGetErrorString(e));
}

#define CK(h, call, what)                                  \
    do {                                                   \
        cudaError_t e_ = (call);                           \
        if (e_ != cudaSuccess) return cuda_err(h, e_, what); \
    } while (0)

int ensure(ebsd_handle* h, DeviceBuf& b, size_t bytes, const char* what)
{
    if (b.bytes >= bytes) return EBSD_OK;
    if (b.ptr) cudaFree(b.ptr);
    b.ptr = nullptr;
    b.bytes = 0;
    cudaError_t e = cudaMalloc(&b.ptr, bytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return set_err(h, EBSD_ENOMEM, "cudaMalloc %zu bytes for %s: %s", bytes, what,
                       cudaGetErrorString(e));
    }
    b.bytes = bytes;
    return EBSD_OK;
}

enum PtrKind { kPageable = 0, kPinned = 1, kDevice = 2 };

PtrKind ptr_kind(const void* p)
{
    cudaPointerAttributes a;
    cudaError_t e = cudaPointerGetAttributes(&a, p);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return kPageable;
    }
    switch (a.type) {
        case cudaMemoryTypeDevice:
        case cudaMemoryTypeManaged: return kDevice;
        case cudaMemoryTypeHost: return kPinned;
        default: return kPageable;
    }
}

// Device memory must belong to the handle's GPU: a kernel launched on
// h->device that dereferences another GPU's memory faults unless peer
// access happens to be enabled, so such pointers are refused before any
// launch.  Managed memory (which migrates) and host memory pass.
int check_device_home(ebsd_handle* h, const char* what, std::initializer_list<const void*> ptrs)
{
    for (const void* p : ptrs) {
        if (!p) continue;
        cudaPointerAttributes a;
        if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
            cudaGetLastError();
            continue;
        }
        if (a.type == cudaMemoryTypeDevice && a.device != h->device)
            return set_err(h, EBSD_EINVAL,
                           "%s: pointer %p is memory of device %d; the handle runs on device %d",
                           what, p, a.device, h->device);
    }
    return EBSD_OK;
}

// Caller device memory that the kernels read or write as float4 (the
// quaternions) must be 16-byte aligned, doubles 8-byte aligned: a
// misaligned vector access would fault, so such pointers are refused.
int check_aligned(ebsd_handle* h, const void* p, size_t a, const char* what)
{
    if (((uintptr_t)p & (a - 1)) != 0)
        return set_err(h, EBSD_EINVAL, "%s: device pointer %p is not %zu-byte aligned", what, p,
                       a);
    return EBSD_OK;
}

int activate(ebsd_handle* h)
{
    CK(h, cudaSetDevice(h->device), "cudaSetDevice");
    return EBSD_OK;
}

// Parallel host copy (pinned staging -> pageable user buffer).
void parallel_memcpy(void* dst, const void* src, size_t bytes)
{
    const size_t min_chunk = size_t(8) << 20;
    unsigned hw = std::thread::hardware_concurrency();
    unsigned nt = (unsigned)std::min<size_t>(std::max(1u, std::min(hw, 16u)),
                                             std::max<size_t>(1, bytes / min_chunk));
    if (nt <= 1) {
        memcpy(dst, src, bytes);
        return;
    }
    std::vector<std::thread> th;
    size_t per = (bytes + nt - 1) / nt;
    per = (per + 63) & ~size_t(63);
    for (unsigned t = 0; t < nt; ++t) {
        size_t off = per * t;
        if (off >= bytes) break;
        size_t n = std::min(per, bytes - off);
        th.emplace_back([=] { memcpy((char*)dst + off, (const char*)src + off, n); });
    }
    for (auto& x : th) x.join();
}

int fill_params(ebsd_handle* h, const ebsd_epilogue* e, FwdParams& p)
{
    memset(&p, 0, sizeof p);
    p.master = h->d_master_il;
    p.rg = h->d_rg;
    p.W = h->d_W;
    p.numsx = h->geom.numsx;
    p.numsy = h->geom.numsy;
    p.P = h->P;
    p.npx = h->npx;
    p.npy = h->npy;
    p.gx = master_pitch(h->npx, h->NV);
    p.scl = host::lambert_scale(h->npx);
    p.spi2 = host::lambert_spi2_f();
    p.accurate = h->lambert_accurate;
    if (h->lambert_accurate == 2 && h->NV > 8)
        return set_err(h, EBSD_EUNSUPPORTED,
                       "lambert_accurate 2 (binary64 geometry): at most 32 energy bins");
    p.rg64 = h->det ? h->det->rg64 : nullptr;
    p.scl64 = (double)h->npx / 1.25331413731550025121;  // npx / sqrt(pi/2)
    p.o_offset = h->noise_offset;
    if (e) {
        if (e->scalingmode < EBSD_SCALING_NOT || e->scalingmode > EBSD_SCALING_GAM)
            return set_err(h, EBSD_EINVAL, "scalingmode %d is not 0 ('not'), 1 ('lin') or 2 ('gam')",
                           e->scalingmode);
        const int b = e->binning;
        if (b != 1 && b != 2 && b != 4 && b != 8)
            return set_err(h, EBSD_EUNSUPPORTED, "binning %d: supported values are 1, 2, 4, 8", b);
        p.prefactor = e->prefactor;
        p.binning = b;
        p.mode = e->scalingmode;
        p.gammavalue = e->gammavalue;
        p.gamma_fast = std::isfinite(e->gammavalue) && e->gammavalue > 0.0f &&
                       e->gammavalue != std::floor(e->gammavalue);
        const float fb = (float)b;
        p.bindx = 1.0f / (fb * fb);
        p.poisson = e->poisson;
        p.seed = e->seed;
        if (p.mode == EBSD_SCALING_NOT || b == 1) {
            p.out_nx = p.numsx;
            p.out_ny = p.numsy;
        } else {
            p.out_nx = p.numsx / b;
            p.out_ny = p.numsy / b;
            if (p.out_nx < 1 || p.out_ny < 1)
                return set_err(h, EBSD_EINVAL, "binning %d leaves no full block on a %dx%d detector",
                               b, p.numsx, p.numsy);
        }
    }
    return EBSD_OK;
}

int check_ready(ebsd_handle* h)
{
    if (!h) return set_err(nullptr, EBSD_EINVAL, "null handle");
    if (!h->have_master) return set_err(h, EBSD_ESTATE, "no master pattern: call ebsd_set_master first");
    if (!h->have_detector)
        return set_err(h, EBSD_ESTATE, "no detector: call ebsd_set_detector first");
    return EBSD_OK;
}

int check_quats_host(ebsd_handle* h, const float* q, int64_t n)
{
    for (int64_t i = 0; i < 4 * n; ++i)
        if (!std::isfinite(q[i]))
            return set_err(h, EBSD_EINVAL, "quaternion %lld has a non-finite component",
                           (long long)(i / 4));
    return EBSD_OK;
}

int launch_chunk(ebsd_handle* h, FwdParams p, const float4* dq, int64_t n, float* dout,
                 int64_t o_offset = 0, bool host_out = false)
{
    p.o_offset += o_offset;
    p.quats = dq;
    p.n = n;
    p.out = dout;
    LaunchCfg cfg = h->cfg;
    if (host_out) cfg.warp_w = 32;  // whole 128-byte rows per warp store into host memory
    cudaError_t e = launch_forward(p, h->NV, cfg, h->stream);
    if (e != cudaSuccess) return cuda_err(h, e, "forward kernel launch");
    return EBSD_OK;
}

}  // namespace

// ----------------------------------------------------------------------

extern "C" int ebsd_version(void) { return 100; }

extern "C" int ebsd_create(ebsd_handle** out, int device)
{
    if (!out) return set_err(nullptr, EBSD_EINVAL, "ebsd_create: null output pointer");
    *out = nullptr;
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return set_err(nullptr, EBSD_ECUDA, "no CUDA device: %s", cudaGetErrorString(e));
    }
    if (device < 0 || device >= ndev)
        return set_err(nullptr, EBSD_EINVAL, "device %d out of range (%d devices)", device, ndev);
    ebsd_handle* h = new ebsd_handle();
    h->device = device;
    e = cudaSetDevice(device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&h->own_stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&h->copy_stream, cudaStreamNonBlocking);
    for (int i = 0; i < 2 && e == cudaSuccess; ++i) {
        e = cudaEventCreateWithFlags(&h->ev_comp[i], cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&h->ev_d2h[i], cudaEventDisableTiming);
    }
    if (e != cudaSuccess) {
        int rc = set_err(nullptr, EBSD_ECUDA, "ebsd_create: %s", cudaGetErrorString(e));
        ebsd_destroy(h);
        return rc;
    }
    h->stream = h->own_stream;
    cudaDeviceGetAttribute(&h->max_persist, cudaDevAttrMaxPersistingL2CacheSize, device);
    cudaDeviceGetAttribute(&h->max_window, cudaDevAttrMaxAccessPolicyWindowSize, device);
    cudaGetLastError();
    *out = h;
    return EBSD_OK;
}

extern "C" void ebsd_destroy(ebsd_handle* h)
{
    if (!h) return;
    cudaSetDevice(h->device);
    if (h->stream) cudaStreamSynchronize(h->stream);
    if (h->copy_stream) cudaStreamSynchronize(h->copy_stream);
    h->ms.reset();
    h->det.reset();
    h->accum.reset();
    cudaSetDevice(h->device);
    cudaFree(h->vjp_partial.ptr);
    cudaFree(h->vjp_io.ptr);
    for (int i = 0; i < 2; ++i) {
        cudaFree(h->quats[i].ptr);
        cudaFree(h->outb[i].ptr);
        if (h->pinned[i]) cudaFreeHost(h->pinned[i]);
        if (h->ev_comp[i]) cudaEventDestroy(h->ev_comp[i]);
        if (h->ev_d2h[i]) cudaEventDestroy(h->ev_d2h[i]);
    }
    cudaFree(h->tmp.ptr);
    cudaFree(h->small.ptr);
    cudaFree(h->wref.ptr);
    cudaFree(h->gn_sys.ptr);
    cudaFree(h->gn_aux.ptr);
    cudaFree(h->batch_table.ptr);
    cudaFree(h->rfz.ptr);
    cudaFree(h->rfz_out.ptr);
    cudaFree(h->mc.ptr);
    if (h->batch_exec) cudaGraphExecDestroy(h->batch_exec);
    if (h->own_stream) cudaStreamDestroy(h->own_stream);
    if (h->copy_stream) cudaStreamDestroy(h->copy_stream);
    cudaGetLastError();
    delete h;
}

extern "C" const char* ebsd_last_error(const ebsd_handle* h)
{
    return h ? h->err.c_str() : g_err.c_str();
}

extern "C" int ebsd_set_stream(ebsd_handle* h, void* stream)
{
    if (!h) return set_err(nullptr, EBSD_EINVAL, "null handle");
    h->stream = stream ? (cudaStream_t)stream : h->own_stream;
    return EBSD_OK;
}

extern "C" int ebsd_set_option(ebsd_handle* h, const char* key, int64_t value)
{
    if (!h) return set_err(nullptr, EBSD_EINVAL, "null handle");
    if (!key) return set_err(h, EBSD_EINVAL, "ebsd_set_option: null key");
    const std::string k(key);
    if (k == "weights_fp64") {
        h->weights_fp64 = value != 0;
        if (h->have_detector)
            return set_err(h, EBSD_ESTATE, "weights_fp64 applies at the next ebsd_set_detector");
    } else if (k == "strict_order") {
        h->cfg.strict = value != 0;

    } else if (k == "l2_persist") {
        if (!value) {
            h->cfg.persist_base = nullptr;
            h->cfg.persist_bytes = 0;
        } else if (!h->cfg.persist_base) {
            return set_err(h, EBSD_ESTATE, "l2_persist: no persisting window on this device/detector");
        }
    } else if (k == "lambert_accurate") {
        if (value < 0 || value > 2)
            return set_err(h, EBSD_EINVAL, "lambert_accurate must be 0, 1 or 2");
        h->lambert_accurate = (int)value;
    } else if (k == "tile_y") {
        if (value != 4 && value != 8 && value != 16)
            return set_err(h, EBSD_EINVAL, "tile_y must be 4, 8 or 16");
        h->cfg.tile_y = (int)value;
    } else if (k == "orient_per_cta") {
        if (value < 0 || value > 64)
            return set_err(h, EBSD_EINVAL, "orient_per_cta must be in 0..64");
        h->cfg.orient_per_cta = (int)value;
    } else if (k == "mc_fp32") {
        h->mc_fp32 = value != 0;
    } else if (k == "host_direct") {
        h->host_direct = value != 0;
    } else if (k == "vjp_tile_y") {
        if (value != 4 && value != 8 && value != 16 && value != 32)
            return set_err(h, EBSD_EINVAL, "vjp_tile_y must be 4, 8, 16 or 32");
        h->vjp_tile_y = (int)value;
    } else if (k == "gn_orient_per_cta") {
        if (value < 1 || value > 64)
            return set_err(h, EBSD_EINVAL, "gn_orient_per_cta must be in 1..64");
        h->gn_opc = (int)value;
    } else if (k == "noise_index_offset") {
        if (value < 0) return set_err(h, EBSD_EINVAL, "noise_index_offset must be >= 0");
        h->noise_offset = value;
    } else if (k == "vjp_orient_per_cta") {
        if (value < 1 || value > 64)
            return set_err(h, EBSD_EINVAL, "vjp_orient_per_cta must be in 1..64");
        h->vjp_opc = (int)value;
    } else {
        return set_err(h, EBSD_EINVAL, "unknown option '%s'", key);
    }
    return EBSD_OK;
}

extern "C" int ebsd_set_master(ebsd_handle* h, const float* sr, int32_t npx, int32_t npy,
                               int32_t nE, int32_t numset)
{
    if (!h) return set_err(nullptr, EBSD_EINVAL, "null handle");
    if (!sr) return set_err(h, EBSD_EINVAL, "ebsd_set_master: null sr");
    if (npx < 1 || npy < 1 || nE < 1 || numset < 1)
        return set_err(h, EBSD_EINVAL, "ebsd_set_master: npx=%d npy=%d nE=%d numset=%d must be >= 1",
                       npx, npy, nE, numset);
    if (nE > 4 * kMaxNV)
        return set_err(h, EBSD_EUNSUPPORTED, "ebsd_set_master: nE=%d exceeds %d energy bins", nE,
                       4 * kMaxNV);
    // the pattern kernels address master nodes with 32-bit offsets
    if ((double)(2 * npx + 8) * (double)(2 * npy + 1) * kMaxNV >= 2147483648.0)
        return set_err(h, EBSD_EUNSUPPORTED,
                       "ebsd_set_master: a %dx%d grid exceeds the 2^31 float4 node offsets",
                       2 * npx + 1, 2 * npy + 1);
    int rc = activate(h);
    if (rc) return rc;
    const size_t n = (size_t)(2 * npx + 1) * (2 * npy + 1) * nE * numset;
    cudaStreamSynchronize(h->stream);
    h->ms.reset();
    h->have_master = false;
    h->have_detector = false;  // window must be rebuilt
    h->d_master_il = nullptr;
    auto ms = std::make_shared<MasterStore>();
    ms->device = h->device;
    CK(h, cudaMalloc(&ms->raw, n * sizeof(float)), "cudaMalloc master");
    CK(h, cudaMemcpy(ms->raw, sr, n * sizeof(float), cudaMemcpyHostToDevice), "master upload");
    ms->npx = npx;
    ms->npy = npy;
    ms->nE = nE;
    ms->numset = numset;
    // maxval(sr) of the set sum, printed by the program (CTEMEBSD.f90:548)
    float mx = -INFINITY;
    const size_t plane = (size_t)(2 * npx + 1) * (2 * npy + 1) * nE;
    for (size_t i = 0; i < plane; ++i) {
        float sum = 0.0f;
        for (int st = 0; st < numset; ++st) sum = sum + sr[i + plane * st];
        mx = std::max(mx, sum);
    }
    ms->max_sr = mx;
    h->ms = std::move(ms);
    h->npx = npx;
    h->npy = npy;
    h->nE = nE;
    h->numset = numset;
    h->have_master = true;
    return EBSD_OK;
}

extern "C" int ebsd_share_master(ebsd_handle* dst, const ebsd_handle* src)
{
    if (!dst || !src) return set_err(dst, EBSD_EINVAL, "ebsd_share_master: null handle");
    if (!src->have_master)
        return set_err(dst, EBSD_ESTATE, "ebsd_share_master: the source handle has no master");
    if (src->device != dst->device)
        return set_err(dst, EBSD_EINVAL, "ebsd_share_master: handles are on devices %d and %d",
                       src->device, dst->device);
    cudaSetDevice(dst->device);
    cudaStreamSynchronize(dst->stream);
    dst->ms = src->ms;
    dst->npx = src->npx;
    dst->npy = src->npy;
    dst->nE = src->nE;
    dst->numset = src->numset;
    dst->have_master = true;
    dst->have_detector = false;
    dst->d_master_il = nullptr;
    return EBSD_OK;
}

extern "C" int ebsd_energy_window(float energymin, float energymax, double Ehistmin,
                                  double Ebinsize, int32_t numEbins, int32_t* Emin, int32_t* Emax)
{
    if (!Emin || !Emax || numEbins < 1 || !(Ebinsize != 0.0))
        return set_err(nullptr, EBSD_EINVAL, "ebsd_energy_window: invalid arguments");
    host::energy_window(energymin, energymax, Ehistmin, Ebinsize, numEbins, Emin, Emax);
    return EBSD_OK;
}

extern "C" double ebsd_prefactor(double beamcurrent, double dwelltime, int32_t num_el)
{
    return host::prefactor(beamcurrent, dwelltime, num_el);
}

namespace {

// Detector tables for geometry g from the histogram already on the device
// (h->accum): direction cosines, weights, derivative tables and, when
// with_num_el, num_el of CTEMEBSD.f90:516.  The energy window and MC grid
// are h's.
int detector_setup(ebsd_handle* h, const ebsd_geometry* g, bool with_num_el)
{
    cudaStream_t s = h->stream;
    CK(h, cudaStreamSynchronize(s), "detector set-up");
    const int P = g->numsx * g->numsy;
    const int nsel = h->Emax - h->Emin + 1;
    const int NV = (nsel + 3) / 4;
    // tables of the right size that no other handle holds (copy on write:
    // a handle sharing them keeps the old ones)
    if (!h->det || h->det.use_count() > 1 || P != h->det->P || NV != h->det->NV) {
        h->d_rg = h->d_W = h->d_drg = h->d_dW = nullptr;
        h->P = 0;
        h->det.reset();
        auto t = std::make_shared<DetectorTables>();
        t->device = h->device;
        CK(h, cudaMalloc(&t->rg, sizeof(float4) * (size_t)P), "cudaMalloc rg");
        CK(h, cudaMalloc(&t->W, sizeof(float4) * (size_t)P * NV), "cudaMalloc W");
        CK(h, cudaMalloc(&t->drg, sizeof(float4) * (size_t)P * 3), "cudaMalloc drg");
        CK(h, cudaMalloc(&t->dW, sizeof(float4) * (size_t)P * (2 * NV + 1)), "cudaMalloc dW");
        CK(h, cudaMalloc(&t->rg64, sizeof(double) * 3 * (size_t)P), "cudaMalloc rg64");
        t->P = P;
        t->NV = NV;
        h->det = std::move(t);
    }
    h->d_rg = h->det->rg;
    h->d_W = h->det->W;
    h->d_drg = h->det->drg;
    h->d_dW = h->det->dW;
    const int32_t* acc = h->accum->ptr;
    float ca, sa;
    host::detector_angles(g->sig, g->thetac, &ca, &sa);
    CK(h, launch_detector(*g, ca, sa, h->d_rg, s), "detector kernel");
    CK(h, launch_detector64(*g, h->det->rg64, s), "binary64 detector kernel");
    const float sclmc = host::lambert_scale(h->nsx);
    // kept by the handle: a refinement of the pattern centre sets the detector
    // up every iteration
    int rcw = ensure(h, h->wref, sizeof(float4) * (size_t)P * NV, "reference weights");
    if (rcw) return rcw;
    float4* d_wref = (float4*)h->wref.ptr;
    cudaError_t e = launch_weights(h->d_rg, P, acc, h->nE, h->nsx, h->nsy, sclmc,
                                   host::lambert_spi2_f(), h->Emin - 1, nsel, NV,
                                   h->weights_fp64, *g, h->d_W, d_wref, s);
    if (e == cudaSuccess)
        e = launch_geom_derivs(*g, acc, h->nE, h->nsx, h->nsy, h->Emin - 1, nsel, NV, h->d_drg,
                               h->d_dW, s);
    float sum = 0.0f;
    if (with_num_el) {
        float* d_sum = (float*)h->small.ptr;
        if (e == cudaSuccess) e = launch_num_el(d_wref, P, nsel, NV, d_sum, s);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(&sum, d_sum, sizeof(float), cudaMemcpyDeviceToHost, s);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_err(h, e, "detector weights");
    if (with_num_el) h->num_el = (int32_t)lroundf(sum);
    h->geom = *g;
    h->P = P;
    h->NV = NV;
    h->nsel = nsel;
    return EBSD_OK;
}

}  // namespace

extern "C" int ebsd_set_detector(ebsd_handle* h, const ebsd_geometry* g, const int32_t* accum_e,
                                 int32_t nsx, int32_t nsy, int32_t numEbins, int32_t Emin,
                                 int32_t Emax, int32_t* num_el)
{
    if (!h) return set_err(nullptr, EBSD_EINVAL, "null handle");
    if (!g || !accum_e) return set_err(h, EBSD_EINVAL, "ebsd_set_detector: null argument");
    if (!h->have_master)
        return set_err(h, EBSD_ESTATE, "ebsd_set_detector: set the master pattern first");
    if (numEbins != h->nE)
        return set_err(h, EBSD_EINVAL,
                       "Energy histogram and Lambert stack have different energy dimension "
                       "(MC numEbins=%d, master nE=%d)",
                       numEbins, h->nE);
    if (g->numsx < 1 || g->numsy < 1 || (int64_t)g->numsx * g->numsy > (1LL << 30))
        return set_err(h, EBSD_EINVAL, "detector %dx%d out of range", g->numsx, g->numsy);
    if (nsx < 1 || nsy < 1) return set_err(h, EBSD_EINVAL, "MC grid nsx=%d nsy=%d", nsx, nsy);
    if (Emin < 1 || Emax > numEbins || Emin > Emax)
        return set_err(h, EBSD_EINVAL, "energy window %d..%d outside 1..%d", Emin, Emax, numEbins);
    if (!(g->L > 0.0f) || !std::isfinite(g->delta) || !std::isfinite(g->xpc) ||
        !std::isfinite(g->ypc) || !std::isfinite(g->thetac) || !std::isfinite(g->sig))
        return set_err(h, EBSD_EINVAL, "detector geometry has a non-finite or non-positive value");
    int rc = activate(h);
    if (rc) return rc;
    cudaStream_t s = h->stream;
    cudaStreamSynchronize(s);
    h->have_detector = false;
    const int nsel = Emax - Emin + 1;
    const int NV = (nsel + 3) / 4;

    // master re-layout for this window
    {
        const auto key = std::make_pair(Emin - 1, nsel);
        auto it = h->ms->layouts.find(key);
        if (it == h->ms->layouts.end()) {
            const size_t bytes =
                sizeof(float4) * (size_t)master_pitch(h->npx, NV) * (2 * h->npy + 1) * NV;
            float4* il = nullptr;
            CK(h, cudaMalloc(&il, bytes), "cudaMalloc master layout");
            cudaError_t e2 = launch_master_relayout(h->ms->raw, h->npx, h->npy, h->nE, h->numset,
                                                    Emin - 1, nsel, NV, il, s);
            if (e2 != cudaSuccess) {
                cudaFree(il);
                return cuda_err(h, e2, "master re-layout");
            }
            it = h->ms->layouts.emplace(key, std::make_pair(il, bytes)).first;
        }
        h->d_master_il = it->second.first;
        h->il_bytes = it->second.second;
    }

    // the histogram stays on the device for later geometry updates (in a
    // store of this handle's own: a shared one is left to its other holders)
    const size_t acc_bytes = sizeof(int32_t) * (size_t)numEbins * (2 * nsx + 1) * (2 * nsy + 1);
    if (!h->accum || h->accum.use_count() > 1 || h->accum->bytes != acc_bytes) {
        h->accum.reset();
        auto a = std::make_shared<HistogramStore>();
        a->device = h->device;
        CK(h, cudaMalloc(&a->ptr, acc_bytes), "cudaMalloc MC histogram");
        a->bytes = acc_bytes;
        h->accum = std::move(a);
    }
    rc = ensure(h, h->small, 256, "set-up scalars");
    if (rc) return rc;
    CK(h, cudaMemcpyAsync(h->accum->ptr, accum_e, acc_bytes, cudaMemcpyHostToDevice, s),
       "MC upload");
    h->Emin = Emin;
    h->Emax = Emax;
    h->nsx = nsx;
    h->nsy = nsy;
    rc = detector_setup(h, g, true);
    if (rc) return rc;
    if (num_el) *num_el = h->num_el;

    // keep the master resident in L2 for the pattern kernels: a persisting
    // carve-out (a limit of this process's context) and an access-policy
    // window attached to every pattern-kernel launch
    h->cfg.persist_base = nullptr;
    h->cfg.persist_bytes = 0;
    if (h->max_persist > 0 && h->max_window > 0) {
        const size_t carve = std::min(h->il_bytes, (size_t)h->max_persist);
        if (cudaDeviceSetLimit(cudaLimitPersistingL2CacheSize, carve) == cudaSuccess) {
            const size_t win = std::min(h->il_bytes, (size_t)h->max_window);
            h->cfg.persist_base = h->d_master_il;
            h->cfg.persist_bytes = win;
            h->cfg.persist_hit_ratio = std::min(1.0f, (float)carve / (float)win);
        }
        cudaGetLastError();
    }
    h->have_detector = true;
    return EBSD_OK;
}

extern "C" int ebsd_share_detector(ebsd_handle* dst, const ebsd_handle* src)
{
    if (!dst || !src) return set_err(dst, EBSD_EINVAL, "ebsd_share_detector: null handle");
    if (dst == src) return EBSD_OK;
    if (!src->have_master || !src->have_detector)
        return set_err(dst, EBSD_ESTATE, "ebsd_share_detector: the source handle has no detector");
    if (src->device != dst->device)
        return set_err(dst, EBSD_EINVAL, "ebsd_share_detector: handles are on devices %d and %d",
                       src->device, dst->device);
    int rc = activate(dst);
    if (rc) return rc;
    // nothing of dst's may still be running on the tables it gives up
    CK(dst, cudaStreamSynchronize(dst->stream), "ebsd_share_detector");
    rc = ensure(dst, dst->small, 256, "set-up scalars");
    if (rc) return rc;
    dst->ms = src->ms;
    dst->npx = src->npx;
    dst->npy = src->npy;
    dst->nE = src->nE;
    dst->numset = src->numset;
    dst->have_master = true;
    dst->d_master_il = src->d_master_il;
    dst->il_bytes = src->il_bytes;
    dst->det = src->det;
    dst->d_rg = src->d_rg;
    dst->d_W = src->d_W;
    dst->d_drg = src->d_drg;
    dst->d_dW = src->d_dW;
    dst->accum = src->accum;
    dst->geom = src->geom;
    dst->Emin = src->Emin;
    dst->Emax = src->Emax;
    dst->nsel = src->nsel;
    dst->NV = src->NV;
    dst->num_el = src->num_el;
    dst->P = src->P;
    dst->nsx = src->nsx;
    dst->nsy = src->nsy;
    dst->weights_fp64 = src->weights_fp64;
    dst->cfg.persist_base = src->cfg.persist_base;
    dst->cfg.persist_bytes = src->cfg.persist_bytes;
    dst->cfg.persist_hit_ratio = src->cfg.persist_hit_ratio;
    dst->have_detector = true;
    return EBSD_OK;
}

extern "C" int ebsd_output_dims(const ebsd_handle* hc, const ebsd_epilogue* e, int32_t* nx,
                                int32_t* ny)
{
    ebsd_handle* h = const_cast<ebsd_handle*>(hc);
    int rc = check_ready(h);
    if (rc) return rc;
    FwdParams p;
    rc = fill_params(h, e, p);
    if (rc) return rc;
    if (nx) *nx = p.out_nx;
    if (ny) *ny = p.out_ny;
    return EBSD_OK;
}

extern "C" int ebsd_forward(ebsd_handle* h, const float* quats, int64_t n, const ebsd_epilogue* e,
                            float* out)
{
    int rc = check_ready(h);
    if (rc) return rc;
    if (n < 0) return set_err(h, EBSD_EINVAL, "negative orientation count");
    if (n == 0) return EBSD_OK;
    if (!quats || !out || !e) return set_err(h, EBSD_EINVAL, "ebsd_forward: null argument");
    rc = check_device_home(h, "ebsd_forward", {quats, out});
    if (rc) return rc;
    rc = activate(h);
    if (rc) return rc;
    FwdParams p;
    rc = fill_params(h, e, p);
    if (rc) return rc;
    const size_t rec = (size_t)p.out_nx * p.out_ny;
    const PtrKind qk = ptr_kind(quats), ok = ptr_kind(out);
    if (qk != kDevice) {
        rc = check_quats_host(h, quats, n);
        if (rc) return rc;
    } else {
        rc = check_aligned(h, quats, 16, "ebsd_forward quats");
        if (rc) return rc;
    }
    cudaStream_t s = h->stream;

    if (ok == kDevice) {
        const float4* dq = (const float4*)quats;
        if (qk != kDevice) {
            rc = ensure(h, h->quats[0], sizeof(float4) * (size_t)n, "quaternions");
            if (rc) return rc;
            CK(h, cudaMemcpyAsync(h->quats[0].ptr, quats, sizeof(float4) * n,
                                  cudaMemcpyHostToDevice, s),
               "quaternion upload");
            dq = (const float4*)h->quats[0].ptr;
        }
        return launch_chunk(h, p, dq, n, out);
    }

    // Pinned host output with host_direct: the kernel stores the records
    // straight into the caller's buffer through its mapped device address
    // (over NVLink-C2C on Grace systems), no staging copy.
    // (the last byte must be pinned too: a kernel store past a mapped region
    // would fault the GPU, where a copy only fails)
    const float* last = out + (size_t)n * rec - 1;
    if (ok == kPinned && h->host_direct && ptr_kind(last) == kPinned) {
        void* dout = nullptr;
        if (cudaHostGetDevicePointer(&dout, out, 0) == cudaSuccess && dout) {
            const float4* dq = (const float4*)quats;
            if (qk != kDevice) {
                rc = ensure(h, h->quats[0], sizeof(float4) * (size_t)n, "quaternions");
                if (rc) return rc;
                CK(h, cudaMemcpyAsync(h->quats[0].ptr, quats, sizeof(float4) * n,
                                      cudaMemcpyHostToDevice, s),
                   "quaternion upload");
                dq = (const float4*)h->quats[0].ptr;
            }
            rc = launch_chunk(h, p, dq, n, (float*)dout, 0, true);
            if (rc) return rc;
            CK(h, cudaStreamSynchronize(s), "forward");
            return EBSD_OK;
        }
        cudaGetLastError();  // not mapped: take the copy path below
    }

    // Host output: chunks of orientations, computed on the work stream and
    // copied back on the copy stream, double-buffered.
    const size_t budget = size_t(256) << 20;
    int64_t chunk = (int64_t)std::max<size_t>(1, budget / (rec * sizeof(float)));
    chunk = std::min<int64_t>(chunk, n);
    const size_t cbytes = (size_t)chunk * rec * sizeof(float);
    for (int b = 0; b < 2; ++b) {
        rc = ensure(h, h->outb[b], cbytes, "pattern chunk");
        if (rc) return rc;
        if (qk != kDevice) {
            rc = ensure(h, h->quats[b], sizeof(float4) * (size_t)chunk, "quaternions");
            if (rc) return rc;
        }
    }
    const bool stage = ok == kPageable;
    if (stage && h->pinned_bytes < cbytes) {
        for (int b = 0; b < 2; ++b) {
            if (h->pinned[b]) cudaFreeHost(h->pinned[b]);
            h->pinned[b] = nullptr;
        }
        h->pinned_bytes = 0;
        for (int b = 0; b < 2; ++b) CK(h, cudaMallocHost(&h->pinned[b], cbytes), "pinned staging");
        h->pinned_bytes = cbytes;
    }
    const int64_t nchunks = (n + chunk - 1) / chunk;
    // fresh events for this call's ordering
    for (int b = 0; b < 2; ++b) CK(h, cudaEventRecord(h->ev_d2h[b], h->copy_stream), "event");
    auto finish = [&](int64_t c) -> int {
        const int b = (int)(c & 1);
        CK(h, cudaEventSynchronize(h->ev_d2h[b]), "pattern copy");
        if (stage) {
            const int64_t o0 = c * chunk;
            const int64_t m = std::min<int64_t>(chunk, n - o0);
            parallel_memcpy(out + (size_t)o0 * rec, h->pinned[b], (size_t)m * rec * sizeof(float));
        }
        return EBSD_OK;
    };
    for (int64_t c = 0; c < nchunks; ++c) {
        const int b = (int)(c & 1);
        const int64_t o0 = c * chunk;
        const int64_t m = std::min<int64_t>(chunk, n - o0);
        if (stage && c >= 2) {
            rc = finish(c - 2);  // staging buffer b must be drained first
            if (rc) return rc;
        }
        CK(h, cudaStreamWaitEvent(s, h->ev_d2h[b], 0), "wait");
        const float4* dq;
        if (qk == kDevice) {
            dq = (const float4*)quats + o0;
        } else {
            CK(h, cudaMemcpyAsync(h->quats[b].ptr, quats + 4 * o0, sizeof(float4) * m,
                                  cudaMemcpyHostToDevice, s),
               "quaternion upload");
            dq = (const float4*)h->quats[b].ptr;
        }
        rc = launch_chunk(h, p, dq, m, (float*)h->outb[b].ptr, o0);
        if (rc) return rc;
        CK(h, cudaEventRecord(h->ev_comp[b], s), "event");
        CK(h, cudaStreamWaitEvent(h->copy_stream, h->ev_comp[b], 0), "wait");
        float* dst = stage ? h->pinned[b] : out + (size_t)o0 * rec;
        CK(h, cudaMemcpyAsync(dst, h->outb[b].ptr, (size_t)m * rec * sizeof(float),
                              cudaMemcpyDeviceToHost, h->copy_stream),
           "pattern copy");
        CK(h, cudaEventRecord(h->ev_d2h[b], h->copy_stream), "event");
    }
    if (stage) {
        for (int64_t c = std::max<int64_t>(0, nchunks - 2); c < nchunks; ++c) {
            rc = finish(c);
            if (rc) return rc;
        }
    } else {
        CK(h, cudaStreamSynchronize(h->copy_stream), "pattern copy");
    }
    // the caller's stream sees completed work
    CK(h, cudaStreamSynchronize(s), "forward");
    return EBSD_OK;
}

extern "C" int ebsd_vjp(ebsd_handle* h, const float* quats, int64_t n, const ebsd_epilogue* e,
                        int32_t mode, const float* data, float* loss, float* grad)
{
    int rc = check_ready(h);
    if (rc) return rc;
    if (n < 0) return set_err(h, EBSD_EINVAL, "negative orientation count");
    if (n == 0) return EBSD_OK;
    if (!quats || !e || !data || !grad) return set_err(h, EBSD_EINVAL, "ebsd_vjp: null argument");
    rc = check_device_home(h, "ebsd_vjp", {quats, data, loss, grad});
    if (rc) return rc;
    if (mode != EBSD_VJP_COTANGENT && mode != EBSD_VJP_NDP)
        return set_err(h, EBSD_EINVAL, "ebsd_vjp: unknown mode %d", mode);
    if (e->scalingmode == EBSD_SCALING_GAM || e->poisson)
        return set_err(h, EBSD_EUNSUPPORTED, "ebsd_vjp: gamma and noise epilogues have no adjoint");
    if (h->NV > 8)
        return set_err(h, EBSD_EUNSUPPORTED, "ebsd_vjp: at most 32 energy bins (window has %d)",
                       h->nsel);
    rc = activate(h);
    if (rc) return rc;
    FwdParams p;
    rc = fill_params(h, e, p);
    if (rc) return rc;
    VjpParams vp;
    memset(&vp, 0, sizeof vp);
    vp.drg = h->d_drg;
    vp.dW = h->d_dW;
    vp.binning = e->scalingmode == EBSD_SCALING_NOT ? 1 : e->binning;
    vp.opc = h->vjp_opc > 0 ? h->vjp_opc : (vp.binning == 1 ? 16 : 8);
    // unbinned records: 32 x 16 tiles by default (tile_y / 4 pixels per
    // thread); binned ones a CTA of 32 x tile_y threads, at most 8 rows
    int tile_y = h->vjp_tile_y > 0 ? h->vjp_tile_y : (vp.binning == 1 ? 16 : 4);
    if (vp.binning > 1) tile_y = vp.binning > std::min(tile_y, 8) ? 8 : std::min(tile_y, 8);
    if (vp.binning > tile_y)
        return set_err(h, EBSD_EUNSUPPORTED, "ebsd_vjp: binning %d exceeds the tile", vp.binning);
    const int K = mode == EBSD_VJP_NDP ? 15 : 6;
    const int ntiles = vjp_tiles(p, tile_y);
    const size_t rec = (size_t)p.out_nx * p.out_ny;
    cudaStream_t s = h->stream;
    const bool qdev = ptr_kind(quats) == kDevice, ddev = ptr_kind(data) == kDevice;
    const bool gdev = ptr_kind(grad) == kDevice;
    const bool ldev = loss ? ptr_kind(loss) == kDevice : true;
    if (!qdev) {
        rc = check_quats_host(h, quats, n);
        if (rc) return rc;
    } else {
        rc = check_aligned(h, quats, 16, "ebsd_vjp quats");
        if (rc) return rc;
    }
    // chunk so that partials and staged records stay bounded
    const size_t budget = size_t(256) << 20;
    const size_t per_o = (size_t)ntiles * K * sizeof(float) + (ddev ? 0 : rec * sizeof(float));
    int64_t chunk = (int64_t)std::max<size_t>(1, budget / per_o);
    chunk = std::min<int64_t>(chunk, n);
    rc = ensure(h, h->vjp_partial, (size_t)chunk * ntiles * K * sizeof(float), "adjoint partials");
    if (rc) return rc;
    // device staging: quats (16 B/o) + data + loss + grad (28 B/o)
    const size_t io_bytes = (size_t)chunk * (16 + 28) + (ddev ? 0 : (size_t)chunk * rec * 4) + 256;
    rc = ensure(h, h->vjp_io, io_bytes, "adjoint staging");
    if (rc) return rc;
    char* io = (char*)h->vjp_io.ptr;
    float4* dq = (float4*)io;
    float* dgrad = (float*)(io + (size_t)chunk * 16);
    float* dloss = dgrad + (size_t)chunk * 6;
    float* ddata = dloss + chunk;
    for (int64_t o0 = 0; o0 < n; o0 += chunk) {
        const int64_t m = std::min<int64_t>(chunk, n - o0);
        p.n = m;
        if (qdev) {
            p.quats = (const float4*)quats + o0;
        } else {
            CK(h, cudaMemcpyAsync(dq, quats + 4 * o0, sizeof(float4) * m, cudaMemcpyHostToDevice, s),
               "quaternion upload");
            p.quats = dq;
        }
        if (ddev) {
            vp.data = data + (size_t)o0 * rec;
        } else {
            CK(h, cudaMemcpyAsync(ddata, data + (size_t)o0 * rec, sizeof(float) * m * rec,
                                  cudaMemcpyHostToDevice, s),
               "record upload");
            vp.data = ddata;
        }
        vp.partial = (float*)h->vjp_partial.ptr;
        vp.grad = gdev ? grad + 6 * o0 : dgrad;
        vp.loss = loss ? (ldev ? loss + o0 : dloss) : nullptr;
        cudaError_t ce = launch_vjp(p, vp, h->NV, mode, tile_y, s);
        if (ce != cudaSuccess) return cuda_err(h, ce, "adjoint kernel launch");
        if (!gdev)
            CK(h, cudaMemcpyAsync(grad + 6 * o0, dgrad, sizeof(float) * 6 * m,
                                  cudaMemcpyDeviceToHost, s),
               "gradient copy");
        if (loss && !ldev)
            CK(h, cudaMemcpyAsync(loss + o0, dloss, sizeof(float) * m, cudaMemcpyDeviceToHost, s),
               "loss copy");
        if (!qdev || !ddev || !gdev || !ldev) CK(h, cudaStreamSynchronize(s), "adjoint");
    }
    return EBSD_OK;
}

// ----------------------------------------------------------------------
// Adjoint without allocation.
//
// Some callers cannot let this library allocate device memory while they
// run the adjoint: a host that owns all GPU memory through its own pool
// (an indexing or refinement framework whose caching allocator must stay
// the only allocator on the device), and a refinement loop that cannot
// afford the device-wide synchronisation cudaMalloc/cudaFree may cause in
// the middle of its iterations.  ebsd_vjp_noalloc serves them: the caller
// passes device buffers for every input and output, and the per-CTA
// partial sums go to the fixed array below instead of a handle-owned
// buffer.  The handle's master and detector tables were allocated earlier,
// by ebsd_set_master / ebsd_set_detector, not by this call.

// 8 MiB of partial sums, resident on every GPU that loads the library until
// the process exits.  One orientation needs ntiles * K floats (ntiles =
// ceil(numsx/32) * ceil(numsy/8), K = 15 in loss mode, 6 in cotangent mode),
// so a 640x480 detector fits 116 orientations per launch; larger batches
// run as several launches through the same array.
constexpr size_t kNoAllocScratchFloats = size_t(2) << 20;
static __device__ __align__(256) float g_vjp_scratch[kNoAllocScratchFloats];

namespace {
constexpr int kMaxDevicesNoAlloc = 64;
std::mutex g_scratch_mu;
float* g_scratch_addr[kMaxDevicesNoAlloc] = {};

// Device address of g_vjp_scratch on the current device (host code may
// only use the symbol through this address).  Looked up once per device, on
// the first call on that device, and kept for the life of the process: a
// cudaDeviceReset, which also destroys every handle's device state, leaves
// the cached address stale, so this entry point must not be used after a
// reset of its device.
int scratch_address(ebsd_handle* h, float** out)
{
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    if (h->device < 0 || h->device >= kMaxDevicesNoAlloc)
        return set_err(h, EBSD_EUNSUPPORTED, "ebsd_vjp_noalloc: device %d beyond %d", h->device,
                       kMaxDevicesNoAlloc);
    if (!g_scratch_addr[h->device]) {
        void* ptr = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&ptr, g_vjp_scratch);
        if (e != cudaSuccess || !ptr) {
            cudaGetLastError();
            return set_err(h, EBSD_ECUDA, "ebsd_vjp_noalloc: scratch address lookup failed: %s",
                           cudaGetErrorString(e));
        }
        g_scratch_addr[h->device] = (float*)ptr;
    }
    *out = g_scratch_addr[h->device];
    return EBSD_OK;
}
}  // namespace

extern "C" int ebsd_vjp_noalloc(ebsd_handle* h, const float* quats, int64_t n,
                                const ebsd_epilogue* e, int32_t mode, const float* data,
                                float* loss, float* grad)
{
    int rc = check_ready(h);
    if (rc) return rc;
    if (n < 0) return set_err(h, EBSD_EINVAL, "negative orientation count");
    if (n == 0) return EBSD_OK;
    if (!quats || !e || !data || !grad)
        return set_err(h, EBSD_EINVAL, "ebsd_vjp_noalloc: null argument");
    if (mode != EBSD_VJP_COTANGENT && mode != EBSD_VJP_NDP)
        return set_err(h, EBSD_EINVAL, "ebsd_vjp_noalloc: unknown mode %d", mode);
    if (e->scalingmode == EBSD_SCALING_GAM || e->poisson)
        return set_err(h, EBSD_EUNSUPPORTED,
                       "ebsd_vjp_noalloc: gamma and noise epilogues have no adjoint");
    if (h->NV > 8)
        return set_err(h, EBSD_EUNSUPPORTED, "ebsd_vjp_noalloc: at most 32 energy bins");
    if (ptr_kind(quats) != kDevice || ptr_kind(data) != kDevice || ptr_kind(grad) != kDevice ||
        (loss && ptr_kind(loss) != kDevice))
        return set_err(h, EBSD_EINVAL,
                       "ebsd_vjp_noalloc: quats, data, loss and grad must be device memory");
    rc = check_device_home(h, "ebsd_vjp_noalloc", {quats, data, loss, grad});
    if (rc) return rc;
    rc = check_aligned(h, quats, 16, "ebsd_vjp_noalloc quats");
    if (rc) return rc;
    rc = activate(h);
    if (rc) return rc;
    float* scratch = nullptr;
    rc = scratch_address(h, &scratch);
    if (rc) return rc;
    FwdParams p;
    rc = fill_params(h, e, p);
    if (rc) return rc;
    VjpParams vp;
    memset(&vp, 0, sizeof vp);
    vp.drg = h->d_drg;
    vp.dW = h->d_dW;
    vp.binning = e->scalingmode == EBSD_SCALING_NOT ? 1 : e->binning;
    vp.opc = 2;
    const int tile_y = 8;
    if (vp.binning > tile_y)
        return set_err(h, EBSD_EUNSUPPORTED, "ebsd_vjp_noalloc: binning %d exceeds the tile",
                       vp.binning);
    const int K = mode == EBSD_VJP_NDP ? 15 : 6;
    const size_t per_o = (size_t)vjp_tiles(p, tile_y) * K;
    if (per_o > kNoAllocScratchFloats)
        return set_err(h, EBSD_EUNSUPPORTED,
                       "ebsd_vjp_noalloc: one orientation of this %dx%d detector needs %zu "
                       "floats of scratch, more than the fixed %zu",
                       p.numsx, p.numsy, per_o, kNoAllocScratchFloats);
    // every partial a launch reads is written by the same launch first, so
    // the array needs no clearing between calls
    const int64_t chunk = (int64_t)(kNoAllocScratchFloats / per_o);
    const size_t rec = (size_t)p.out_nx * p.out_ny;
    for (int64_t o0 = 0; o0 < n; o0 += chunk) {
        const int64_t m = std::min<int64_t>(chunk, n - o0);
        p.n = m;
        p.quats = (const float4*)quats + o0;
        vp.data = data + (size_t)o0 * rec;
        vp.partial = scratch;
        vp.grad = grad + 6 * o0;
        vp.loss = loss ? loss + o0 : nullptr;
        cudaError_t ce = launch_vjp(p, vp, h->NV, mode, tile_y, h->stream);
        if (ce != cudaSuccess) return cuda_err(h, ce, "ebsd_vjp_noalloc launch");
    }
    return EBSD_OK;
}


// ----------------------------------------------------------------------
// Gauss-Newton refinement

namespace {

int gn_check(ebsd_handle* h, const ebsd_epilogue* e, const float* quats, const float* targets)
{
    if (!e || !quats || !targets) return set_err(h, EBSD_EINVAL, "Gauss-Newton: null argument");
    if (e->scalingmode == EBSD_SCALING_GAM || e->poisson)
        return set_err(h, EBSD_EUNSUPPORTED, "Gauss-Newton: gamma and noise have no adjoint");
    if (h->NV > 8) return set_err(h, EBSD_EUNSUPPORTED, "Gauss-Newton: at most 32 energy bins");
    if (ptr_kind(quats) != kDevice || ptr_kind(targets) != kDevice)
        return set_err(h, EBSD_EINVAL, "Gauss-Newton: quats and targets must be device memory");
    const int rc = check_device_home(h, "Gauss-Newton", {quats, targets});
    if (rc) return rc;
    return check_aligned(h, quats, 16, "Gauss-Newton quats");
}

}  // namespace

extern "C" int ebsd_gn_accumulate(ebsd_handle* h, const float* quats, int64_t n,
                                  const ebsd_epilogue* e, const float* targets, double damping,
                                  double* pc_system, float* loss)
{
    int rc = check_ready(h);
    if (rc) return rc;
    if (n < 1) return set_err(h, EBSD_EINVAL, "ebsd_gn_accumulate: no orientations");
    rc = gn_check(h, e, quats, targets);
    if (rc) return rc;
    if (loss && ptr_kind(loss) != kDevice)
        return set_err(h, EBSD_EINVAL, "ebsd_gn_accumulate: loss must be device memory");
    rc = check_device_home(h, "ebsd_gn_accumulate", {loss});
    if (rc) return rc;
    rc = activate(h);
    if (rc) return rc;
    FwdParams p;
    rc = fill_params(h, e, p);
    if (rc) return rc;
    VjpParams vp;
    memset(&vp, 0, sizeof vp);
    vp.drg = h->d_drg;
    vp.dW = h->d_dW;
    vp.binning = e->scalingmode == EBSD_SCALING_NOT ? 1 : e->binning;
    vp.opc = h->gn_opc;
    // records binned 2x2 or 4x4: 32 x 16 tiles by default (four pixel rows
    // per thread); otherwise a CTA of 32 x tile_y threads, at most 8 rows
    int tile_y;
    if (vp.binning == 2 || vp.binning == 4) {
        tile_y = h->vjp_tile_y > 0 ? h->vjp_tile_y : 16;
    } else {
        const int ty_opt = h->vjp_tile_y > 0 ? std::min(h->vjp_tile_y, 8) : 4;
        tile_y = vp.binning > ty_opt ? 8 : ty_opt;
    }
    if (vp.binning > tile_y)
        return set_err(h, EBSD_EUNSUPPORTED, "Gauss-Newton: binning %d exceeds the tile",
                       vp.binning);
    const int ntiles = vjp_tiles(p, tile_y);
    const size_t rec = (size_t)p.out_nx * p.out_ny;
    const size_t per_o = (size_t)ntiles * kGnPartialK * sizeof(float);
    int64_t chunk = (int64_t)std::max<size_t>(1, (size_t(512) << 20) / per_o);
    chunk = std::min<int64_t>(chunk, n);
    rc = ensure(h, h->vjp_partial, (size_t)chunk * per_o, "Gauss-Newton partials");
    if (rc) return rc;
    rc = ensure(h, h->gn_sys, sizeof(double) * kGnSysK * (size_t)n, "Gauss-Newton systems");
    if (rc) return rc;
    const int nb = gn_schur_blocks(n);
    const size_t aux = sizeof(double) * (12 * (size_t)nb + 12 + 4) + sizeof(float) * (size_t)n;
    rc = ensure(h, h->gn_aux, aux, "Gauss-Newton scratch");
    if (rc) return rc;
    cudaStream_t s = h->stream;
    double* sys = (double*)h->gn_sys.ptr;
    for (int64_t o0 = 0; o0 < n; o0 += chunk) {
        const int64_t m = std::min<int64_t>(chunk, n - o0);
        p.n = m;
        p.quats = (const float4*)quats + o0;
        vp.data = targets + (size_t)o0 * rec;
        vp.partial = (float*)h->vjp_partial.ptr;
        cudaError_t ce = launch_gn_accumulate(p, vp, h->NV, tile_y, sys + kGnSysK * o0,
                                              loss ? loss + o0 : nullptr, s);
        if (ce != cudaSuccess) return cuda_err(h, ce, "Gauss-Newton accumulate");
    }
    h->gn_n = n;
    if (pc_system) {
        double* partial = (double*)h->gn_aux.ptr;
        double* out = partial + 12 * (size_t)nb;
        CK(h, launch_gn_schur(sys, n, damping, partial, out, s), "Gauss-Newton centre system");
        CK(h, cudaMemcpyAsync(pc_system, out, 12 * sizeof(double), cudaMemcpyDeviceToHost, s),
           "centre system copy");
        CK(h, cudaStreamSynchronize(s), "Gauss-Newton accumulate");
    }
    return EBSD_OK;
}

extern "C" int ebsd_gn_apply(ebsd_handle* h, float* quats, int64_t n, double damping,
                             const double* dpc, double* max_step)
{
    int rc = check_ready(h);
    if (rc) return rc;
    if (n != h->gn_n || n < 1)
        return set_err(h, EBSD_ESTATE, "ebsd_gn_apply: %lld orientations, the last accumulate "
                       "had %lld", (long long)n, (long long)h->gn_n);
    if (!quats || ptr_kind(quats) != kDevice)
        return set_err(h, EBSD_EINVAL, "ebsd_gn_apply: quats must be device memory");
    rc = check_device_home(h, "ebsd_gn_apply", {quats});
    if (rc) return rc;
    rc = check_aligned(h, quats, 16, "ebsd_gn_apply quats");
    if (rc) return rc;
    rc = activate(h);
    if (rc) return rc;
    cudaStream_t s = h->stream;
    const int nb = gn_schur_blocks(n);
    double* d_dpc = (double*)h->gn_aux.ptr + 12 * (size_t)nb + 12;
    float* steps = (float*)(d_dpc + 4);
    if (dpc) CK(h, cudaMemcpyAsync(d_dpc, dpc, 3 * sizeof(double), cudaMemcpyHostToDevice, s),
                "centre step upload");
    CK(h, launch_gn_update((const double*)h->gn_sys.ptr, n, damping, dpc ? d_dpc : nullptr,
                           (float4*)quats, steps, s),
       "Gauss-Newton update");
    if (max_step) {
        std::vector<float> st((size_t)n);
        CK(h, cudaMemcpyAsync(st.data(), steps, sizeof(float) * n, cudaMemcpyDeviceToHost, s),
           "step copy");
        CK(h, cudaStreamSynchronize(s), "Gauss-Newton apply");
        double mx = 0.0;
        for (float v : st) mx = std::max(mx, (double)v);
        *max_step = mx;
    }
    return EBSD_OK;
}

// Solve the damped 3x3 centre system (S + lambda diag S) d = r.
static bool solve3(const double S[9], const double r[3], double lambda, double d[3])
{
    double A[9];
    memcpy(A, S, sizeof A);
    for (int i = 0; i < 3; ++i) A[i * 4] *= 1.0 + lambda;
    const double c00 = A[4] * A[8] - A[5] * A[7], c01 = A[5] * A[6] - A[3] * A[8],
                 c02 = A[3] * A[7] - A[4] * A[6];
    const double det = A[0] * c00 + A[1] * c01 + A[2] * c02;
    if (!(std::fabs(det) > 0.0) || !std::isfinite(det)) return false;
    const double inv[9] = {c00, A[2] * A[7] - A[1] * A[8], A[1] * A[5] - A[2] * A[4],
                           c01, A[0] * A[8] - A[2] * A[6], A[2] * A[3] - A[0] * A[5],
                           c02, A[1] * A[6] - A[0] * A[7], A[0] * A[4] - A[1] * A[3]};
    for (int i = 0; i < 3; ++i)
        d[i] = (inv[i * 3] * r[0] + inv[i * 3 + 1] * r[1] + inv[i * 3 + 2] * r[2]) / det;
    return true;
}

extern "C" int ebsd_refine(ebsd_handle* h, float* quats, int64_t n, const ebsd_epilogue* e,
                           const float* targets, const ebsd_gn_options* opt, float* loss,
                           ebsd_geometry* geom, int32_t* iterations)
{
    int rc = check_ready(h);
    if (rc) return rc;
    if (!opt || opt->max_iterations < 0) return set_err(h, EBSD_EINVAL, "ebsd_refine: options");
    if (opt->refine_pc && !geom)
        return set_err(h, EBSD_EINVAL, "ebsd_refine: refine_pc needs the geometry argument");
    int it = 0;
    ebsd_geometry g = h->geom;
    for (; it < opt->max_iterations; ++it) {
        double sysc[12];
        rc = ebsd_gn_accumulate(h, quats, n, e, targets, opt->damping,
                                opt->refine_pc ? sysc : nullptr, loss);
        if (rc) return rc;
        double dpc[3] = {0.0, 0.0, 0.0};
        if (opt->refine_pc && !solve3(sysc, sysc + 9, opt->damping, dpc))
            dpc[0] = dpc[1] = dpc[2] = 0.0;
        double mstep = 0.0;
        rc = ebsd_gn_apply(h, quats, n, opt->damping, opt->refine_pc ? dpc : nullptr, &mstep);
        if (rc) return rc;
        const double pcstep = std::max(std::fabs(dpc[0]), std::max(std::fabs(dpc[1]),
                                                                   std::fabs(dpc[2])));
        if (opt->refine_pc && pcstep > 0.0) {
            g.xpc = (float)((double)g.xpc + dpc[0]);
            g.ypc = (float)((double)g.ypc + dpc[1]);
            g.L = (float)((double)g.L + dpc[2]);
            rc = detector_setup(h, &g, false);
            if (rc) return rc;
        }
        if (mstep < opt->tol_rad && (!opt->refine_pc || pcstep < opt->tol_pc)) {
            ++it;
            break;
        }
    }
    if (loss) {  // loss at the final estimate
        rc = ebsd_gn_accumulate(h, quats, n, e, targets, opt->damping, nullptr, loss);
        if (rc) return rc;
        CK(h, cudaStreamSynchronize(h->stream), "refine");
    }
    if (geom) *geom = h->geom;
    if (iterations) *iterations = it;
    return EBSD_OK;
}

extern "C" int ebsd_refine_sharded(ebsd_handle* const* hs, int32_t nh, float* const* quats,
                                   const int64_t* n, const ebsd_epilogue* e,
                                   const float* const* targets, const ebsd_gn_options* opt,
                                   float* const* loss, ebsd_geometry* geom, int32_t* iterations)
{
    if (!hs || nh < 1 || nh > 64 || !quats || !n || !targets)
        return set_err(nullptr, EBSD_EINVAL, "ebsd_refine_sharded: bad handle or shard lists");
    ebsd_handle* h0 = hs[0];
    for (int k = 0; k < nh; ++k) {
        int rc = check_ready(hs[k]);
        if (rc) return rc;
        if (hs[k]->geom.numsx != h0->geom.numsx || hs[k]->geom.numsy != h0->geom.numsy ||
            memcmp(&hs[k]->geom, &h0->geom, sizeof(ebsd_geometry)) != 0)
            return set_err(h0, EBSD_EINVAL, "ebsd_refine_sharded: handle %d has another detector "
                           "geometry than handle 0", k);
        for (int j = 0; j < k; ++j)
            if (hs[j] == hs[k])
                return set_err(h0, EBSD_EINVAL, "ebsd_refine_sharded: handle %d listed twice", k);
    }
    if (!opt || opt->max_iterations < 0)
        return set_err(h0, EBSD_EINVAL, "ebsd_refine_sharded: options");
    if (opt->refine_pc && !geom)
        return set_err(h0, EBSD_EINVAL, "ebsd_refine_sharded: refine_pc needs the geometry");
    // run f(k) for every shard with orientations, each on its own host thread;
    // the first failing shard's message goes to handle 0
    std::vector<int> rcs(nh, EBSD_OK);
    auto each = [&](auto f) -> int {
        std::vector<std::thread> th;
        for (int k = 0; k < nh; ++k)
            if (n[k] > 0) th.emplace_back([&, k] { rcs[k] = f(k); });
        for (auto& t : th) t.join();
        for (int k = 0; k < nh; ++k)
            if (rcs[k]) {
                if (k) set_err(h0, rcs[k], "shard %d: %s", k, std::string(hs[k]->err).c_str());
                return rcs[k];
            }
        return EBSD_OK;
    };
    std::vector<double> sys((size_t)nh * 12), steps(nh);
    ebsd_geometry g = h0->geom;
    int it = 0, rc = EBSD_OK;
    for (; it < opt->max_iterations; ++it) {
        rc = each([&](int k) {
            return ebsd_gn_accumulate(hs[k], quats[k], n[k], e, targets[k], opt->damping,
                                      opt->refine_pc ? &sys[12 * k] : nullptr,
                                      loss ? loss[k] : nullptr);
        });
        if (rc) return rc;
        // the pattern-centre system: the sum over shards, in shard order
        double sum[12] = {0.0};
        for (int k = 0; k < nh; ++k)
            if (n[k] > 0)
                for (int i = 0; i < 12; ++i) sum[i] += sys[12 * k + i];
        double dpc[3] = {0.0, 0.0, 0.0};
        if (opt->refine_pc && !solve3(sum, sum + 9, opt->damping, dpc))
            dpc[0] = dpc[1] = dpc[2] = 0.0;
        rc = each([&](int k) {
            return ebsd_gn_apply(hs[k], quats[k], n[k], opt->damping,
                                 opt->refine_pc ? dpc : nullptr, &steps[k]);
        });
        if (rc) return rc;
        double mstep = 0.0;
        for (int k = 0; k < nh; ++k)
            if (n[k] > 0) mstep = std::max(mstep, steps[k]);
        const double pcstep = std::max(std::fabs(dpc[0]), std::max(std::fabs(dpc[1]),
                                                                   std::fabs(dpc[2])));
        if (opt->refine_pc && pcstep > 0.0) {
            g.xpc = (float)((double)g.xpc + dpc[0]);
            g.ypc = (float)((double)g.ypc + dpc[1]);
            g.L = (float)((double)g.L + dpc[2]);
            for (int k = 0; k < nh; ++k) {  // every handle, including idle shards
                rc = activate(hs[k]);
                if (!rc) rc = detector_setup(hs[k], &g, false);
                if (rc) {
                    if (k) set_err(h0, rc, "shard %d: %s", k, std::string(hs[k]->err).c_str());
                    return rc;
                }
            }
        }
        if (mstep < opt->tol_rad && (!opt->refine_pc || pcstep < opt->tol_pc)) {
            ++it;
            break;
        }
    }
    if (loss) {  // loss at the final estimate
        rc = each([&](int k) {
            int r = ebsd_gn_accumulate(hs[k], quats[k], n[k], e, targets[k], opt->damping,
                                       nullptr, loss[k]);
            if (!r && cudaStreamSynchronize(hs[k]->stream) != cudaSuccess)
                r = cuda_err(hs[k], cudaGetLastError(), "refine");
            return r;
        });
        if (rc) return rc;
    }
    if (geom) *geom = h0->geom;
    if (iterations) *iterations = it;
    return EBSD_OK;
}

// ----------------------------------------------------------------------
// Batched pattern loop

namespace {

struct BatchGroup {
    int NV;
    bool noise;
    int ty;     // tile height of the group's launch
    bool bin8;  // 8x8-binned records
    std::vector<BatchJob> jobs;
};

// A job that fills the GPU by itself: launched on its own, at its handle's
// (tuned) launch shape, inside the batch's stream or graph.
struct BatchLarge {
    FwdParams p;
    int NV;
    LaunchCfg cfg;
};

// A job whose own launch has at least this many CTAs per SM (several full
// waves) runs as its own launch; smaller ones share the persistent queue.
constexpr int kBatchLargeCtasPerSm = 64;

}  // namespace

extern "C" int ebsd_forward_batched(ebsd_handle* h, const ebsd_job* jobs, int32_t njobs,
                                    int32_t flags)
{
    if (!h) return set_err(nullptr, EBSD_EINVAL, "null handle");
    if (njobs < 0 || (njobs > 0 && !jobs))
        return set_err(h, EBSD_EINVAL, "ebsd_forward_batched: bad job list");
    int rc = activate(h);
    if (rc) return rc;
    int sms = 1;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, h->device);
    std::vector<BatchGroup> groups;
    std::vector<BatchLarge> large;
    for (int j = 0; j < njobs; ++j) {
        const ebsd_job& J = jobs[j];
        ebsd_handle* src = J.source;
        if (!src || !src->have_master || !src->have_detector)
            return set_err(h, EBSD_ESTATE, "job %d: source handle has no master/detector", j);
        if (src->device != h->device)
            return set_err(h, EBSD_EINVAL, "job %d is on device %d, the batch runs on %d", j,
                           src->device, h->device);
        if (J.n < 0) return set_err(h, EBSD_EINVAL, "job %d: negative orientation count", j);
        if (J.n == 0) continue;
        if (!J.quats || !J.out) return set_err(h, EBSD_EINVAL, "job %d: null pointer", j);
        if (ptr_kind(J.quats) != kDevice || ptr_kind(J.out) != kDevice)
            return set_err(h, EBSD_EINVAL, "job %d: quats and out must be device memory", j);
        if (check_device_home(h, "ebsd_forward_batched", {J.quats, J.out}))
            return set_err(h, EBSD_EINVAL, "job %d: %s", j, std::string(h->err).c_str());
        if (((uintptr_t)J.quats & 15) != 0)
            return set_err(h, EBSD_EINVAL, "job %d: quats not 16-byte aligned", j);
        if (src->NV > 8)
            return set_err(h, EBSD_EUNSUPPORTED, "job %d: more than 32 energy bins", j);
        BatchJob b;
        memset(&b, 0, sizeof b);
        rc = fill_params(src, &J.epilogue, b.p);
        if (rc) return set_err(h, rc, "job %d: %s", j, src->err.c_str());
        b.p.quats = (const float4*)J.quats;
        b.p.out = J.out;
        b.p.n = J.n;
        // the binary64-geometry mode exists only in the per-job pattern kernel
        if (b.p.accurate == 2 ||
            (!(flags & EBSD_BATCH_QUEUE_ALL) &&
             forward_ctas(b.p, src->cfg) >= (int64_t)kBatchLargeCtasPerSm * sms)) {
            BatchLarge L;
            memset(&L, 0, sizeof L);
            L.p = b.p;
            L.NV = src->NV;
            L.cfg = src->cfg;
            large.push_back(L);
            continue;
        }
        // the job's tuned tile height, raised until binned records hold whole
        // blocks, as its own launch would run it
        int ty = src->cfg.tile_y;
        const bool binned = b.p.mode != EBSD_SCALING_NOT && b.p.binning > 1;
        if (binned)
            while (ty % b.p.binning != 0 && ty < 16) ty *= 2;
        const bool bin8 = binned && b.p.binning == 8;
        if (!batch_shape_ok(ty, bin8))
            return set_err(h, EBSD_EINVAL, "job %d: tile height %d", j, ty);
        b.tiles_x = (b.p.numsx + kTileX - 1) / kTileX;
        b.ntiles = b.tiles_x * ((b.p.numsy + ty - 1) / ty);
        // items of 32 x ty pixels x opc orientations, >= 4096 pixel-patterns:
        // each item costs a barrier, a queue claim and its tile's weight
        // loads (64-job uneven workload: 214 k patterns/s against 204 k with
        // 1024-pixel-pattern items)
        b.opc = std::max(128 / ty, src->cfg.orient_per_cta);
        b.items = (long long)b.ntiles * ((J.n + b.opc - 1) / b.opc);
        const bool noise = J.epilogue.poisson != 0;
        auto g = std::find_if(groups.begin(), groups.end(), [&](const BatchGroup& x) {
            return x.NV == src->NV && x.noise == noise && x.ty == ty && x.bin8 == bin8;
        });
        if (g == groups.end()) {
            groups.push_back({src->NV, noise, ty, bin8, {}});
            g = groups.end() - 1;
        }
        g->jobs.push_back(b);
    }
    if (groups.empty() && large.empty()) return EBSD_OK;
    std::sort(groups.begin(), groups.end(), [](const BatchGroup& a, const BatchGroup& b) {
        if (a.NV != b.NV) return a.NV < b.NV;
        if (a.noise != b.noise) return a.noise < b.noise;
        if (a.ty != b.ty) return a.ty < b.ty;
        return a.bin8 < b.bin8;
    });

    // launches of the queue kernel: each group's jobs in chunks of at most
    // kBatchLaunchJobs, each chunk a launch with its own queue counter and
    // its jobs in the kernel parameters
    struct QueueLaunch {
        size_t group;
        std::unique_ptr<BatchLaunch> table;
        int grid;
    };
    std::vector<QueueLaunch> qls;
    for (size_t gi = 0; gi < groups.size(); ++gi) {
        auto& g = groups[gi];
        const int gk = g.NV * 128 + (g.noise ? 64 : 0) + (g.bin8 ? 32 : 0) + g.ty;
        auto it = h->batch_grid.find(gk);
        if (it == h->batch_grid.end())
            it = h->batch_grid.emplace(gk, batched_grid(g.NV, g.noise, g.ty, g.bin8)).first;
        for (size_t j0 = 0; j0 < g.jobs.size(); j0 += kBatchLaunchJobs) {
            const size_t nj = std::min(g.jobs.size() - j0, (size_t)kBatchLaunchJobs);
            auto L = std::make_unique<BatchLaunch>();
            memset(L.get(), 0, sizeof(BatchLaunch));
            long long begin = 0;
            for (size_t j = 0; j < nj; ++j) {
                L->job[j] = g.jobs[j0 + j];
                L->job[j].item_begin = begin;
                begin += L->job[j].items;
            }
            L->total_items = begin;
            L->njobs = (int)nj;
            qls.push_back({gi, std::move(L), it->second});
        }
    }
    const size_t NQ = qls.size();

    // (the counters are reset in stream order, so an earlier batch still in
    // flight on this stream is not disturbed)
    // a graph bakes every launch's parameters into its kernel nodes: it is
    // reused only for an identical job list (the same buffers and sizes)
    std::vector<int> key;
    for (auto& q : qls) {
        const auto& g = groups[q.group];
        key.push_back(g.NV * 128 + (g.noise ? 64 : 0) + (g.bin8 ? 32 : 0) + g.ty);
        const int* w = reinterpret_cast<const int*>(q.table.get());  // zero-filled padding
        key.insert(key.end(), w, w + (16 + q.table->njobs * sizeof(BatchJob)) / sizeof(int));
    }
    for (auto& L : large) {
        key.push_back(-1);
        const int* w = reinterpret_cast<const int*>(&L.p);  // zero-filled padding
        key.insert(key.end(), w, w + sizeof(FwdParams) / sizeof(int));
        const uint64_t pb = (uint64_t)(uintptr_t)L.cfg.persist_base;
        int hr;
        memcpy(&hr, &L.cfg.persist_hit_ratio, sizeof hr);
        key.insert(key.end(), {L.NV, L.cfg.tile_y, L.cfg.orient_per_cta, L.cfg.warp_w,
                               (int)L.cfg.strict, (int)(pb >> 32), (int)pb,
                               (int)(L.cfg.persist_bytes >> 32), (int)L.cfg.persist_bytes, hr});
    }
    const bool use_graph = (flags & EBSD_BATCH_GRAPH) != 0;
    const bool reuse = use_graph && h->batch_exec && h->batch_key == key &&
                       h->batch_stream == h->stream;
    if (!reuse) {
        if (h->batch_exec) {
            cudaGraphExecDestroy(h->batch_exec);
            h->batch_exec = nullptr;
        }
    }
    if (NQ > 0) {
        rc = ensure(h, h->batch_table, NQ * sizeof(unsigned long long), "batch queue counters");
        if (rc) return rc;
    }
    unsigned long long* counters = (unsigned long long*)h->batch_table.ptr;
    cudaStream_t s = h->stream;
    auto enqueue = [&]() -> cudaError_t {
        cudaError_t e = cudaSuccess;
        for (size_t i = 0; i < large.size() && e == cudaSuccess; ++i)
            e = launch_forward(large[i].p, large[i].NV, large[i].cfg, s);
        if (NQ == 0) return e;
        if (e == cudaSuccess) e = cudaMemsetAsync(counters, 0, NQ * sizeof(unsigned long long), s);
        for (size_t i = 0; i < NQ && e == cudaSuccess; ++i) {
            const auto& g = groups[qls[i].group];
            e = launch_forward_batched(*qls[i].table, counters + i, g.NV, g.noise, g.ty, g.bin8,
                                       qls[i].grid, s);
        }
        return e;
    };
    if (!use_graph) {
        cudaError_t e = enqueue();
        if (e != cudaSuccess) return cuda_err(h, e, "batched launch");
        return EBSD_OK;
    }
    if (!reuse) {
        cudaGraph_t graph = nullptr;
        CK(h, cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal), "graph capture");
        cudaError_t e = enqueue();
        cudaError_t e2 = cudaStreamEndCapture(s, &graph);
        if (e != cudaSuccess || e2 != cudaSuccess) {
            if (graph) cudaGraphDestroy(graph);
            return cuda_err(h, e != cudaSuccess ? e : e2, "graph capture");
        }
        e = cudaGraphInstantiate(&h->batch_exec, graph, 0);
        cudaGraphDestroy(graph);
        if (e != cudaSuccess) {
            h->batch_exec = nullptr;
            return cuda_err(h, e, "graph instantiate");
        }
        h->batch_key = key;
        h->batch_stream = s;
    }
    CK(h, cudaGraphLaunch(h->batch_exec, s), "graph launch");
    return EBSD_OK;
}

// ----------------------------------------------------------------------
// Launch-shape autotuner

namespace {

std::string tune_key(ebsd_handle* h, const FwdParams& p)
{
    int sms = 0, major = 0, minor = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, h->device);
    cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, h->device);
    cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, h->device);
    char buf[256];
    snprintf(buf, sizeof buf, "sm%d%d_x%d det%dx%d nv%d bin%d mode%d strict%d acc%d", major, minor,
             sms, p.numsx, p.numsy, h->NV, p.binning, p.mode, (int)h->cfg.strict, p.accurate);
    return buf;
}

bool tune_lookup(const char* path, const std::string& key, int* ty, int* opc, float* us)
{
    if (!path) return false;
    FILE* f = fopen(path, "r");
    if (!f) return false;
    char line[512];
    bool found = false;
    while (fgets(line, sizeof line, f)) {
        char* bar = strchr(line, '|');
        if (!bar) continue;
        *bar = 0;
        if (key != line) continue;
        int a, b;
        float c;
        if (sscanf(bar + 1, "%d|%d|%f", &a, &b, &c) == 3) {
            *ty = a;
            *opc = b;
            *us = c;
            found = true;  // the last entry for a key wins
        }
    }
    fclose(f);
    return found;
}

}  // namespace

extern "C" int ebsd_autotune(ebsd_handle* h, const ebsd_epilogue* e, int64_t n_sample,
                             const char* cache_path, int32_t* tile_y, int32_t* opc,
                             float* us_per_pattern)
{
    int rc = check_ready(h);
    if (rc) return rc;
    if (!e || n_sample < 1) return set_err(h, EBSD_EINVAL, "ebsd_autotune: invalid arguments");
    rc = activate(h);
    if (rc) return rc;
    FwdParams p;
    rc = fill_params(h, e, p);
    if (rc) return rc;
    const std::string key = tune_key(h, p);
    int best_ty = 0, best_opc = 0;
    float best_us = 0.0f;
    if (!tune_lookup(cache_path, key, &best_ty, &best_opc, &best_us)) {
        // sample orientations: a fixed pseudo-random set of unit quaternions
        std::vector<float> q(4 * (size_t)n_sample);
        uint64_t st = 0x9E3779B97F4A7C15ull;
        auto rnd = [&]() {
            st ^= st << 13;
            st ^= st >> 7;
            st ^= st << 17;
            return (double)(st >> 11) * (1.0 / 9007199254740992.0);
        };
        for (int64_t i = 0; i < n_sample; ++i) {
            const double u1 = rnd(), u2 = rnd(), u3 = rnd();
            const double a = std::sqrt(1.0 - u1), b = std::sqrt(u1);
            q[4 * i + 0] = (float)(b * std::cos(2 * M_PI * u3));
            q[4 * i + 1] = (float)(a * std::sin(2 * M_PI * u2));
            q[4 * i + 2] = (float)(a * std::cos(2 * M_PI * u2));
            q[4 * i + 3] = (float)(b * std::sin(2 * M_PI * u3));
        }
        const size_t rec = (size_t)p.out_nx * p.out_ny;
        float4* dq = nullptr;
        float* dout = nullptr;
        cudaEvent_t e0 = nullptr, e1 = nullptr;
        cudaError_t ce = cudaMalloc(&dq, sizeof(float4) * n_sample);
        if (ce == cudaSuccess) ce = cudaMalloc(&dout, sizeof(float) * rec * n_sample);
        if (ce == cudaSuccess)
            ce = cudaMemcpy(dq, q.data(), sizeof(float4) * n_sample, cudaMemcpyHostToDevice);
        if (ce == cudaSuccess) ce = cudaEventCreate(&e0);
        if (ce == cudaSuccess) ce = cudaEventCreate(&e1);
        const LaunchCfg saved = h->cfg;
        p.quats = dq;
        p.out = dout;
        p.n = n_sample;
        best_us = INFINITY;
        const int tys[3] = {4, 8, 16};
        const int opcs[7] = {1, 2, 4, 8, 16, 32, 64};
        for (int ty : tys) {
            if (ce != cudaSuccess) break;
            if (p.binning > 1 && p.mode != EBSD_SCALING_NOT && ty % p.binning != 0) continue;
            for (int oc : opcs) {
                h->cfg.tile_y = ty;
                h->cfg.orient_per_cta = oc;
                ce = launch_forward(p, h->NV, h->cfg, h->stream);  // warm-up
                if (ce != cudaSuccess) break;
                ce = cudaEventRecord(e0, h->stream);
                for (int r = 0; r < 3 && ce == cudaSuccess; ++r)
                    ce = launch_forward(p, h->NV, h->cfg, h->stream);
                if (ce == cudaSuccess) ce = cudaEventRecord(e1, h->stream);
                if (ce == cudaSuccess) ce = cudaEventSynchronize(e1);
                float ms = 0.0f;
                if (ce == cudaSuccess) ce = cudaEventElapsedTime(&ms, e0, e1);
                if (ce != cudaSuccess) break;
                const float us = 1000.0f * ms / (3.0f * (float)n_sample);
                if (us < best_us) {
                    best_us = us;
                    best_ty = ty;
                    best_opc = oc;
                }
            }
        }
        h->cfg = saved;
        cudaFree(dq);
        cudaFree(dout);
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
        if (ce != cudaSuccess) return cuda_err(h, ce, "ebsd_autotune");
        if (cache_path) {
            FILE* f = fopen(cache_path, "a");
            if (f) {
                fprintf(f, "%s|%d|%d|%.4f\n", key.c_str(), best_ty, best_opc, best_us);
                fclose(f);
            }
        }
    }
    h->cfg.tile_y = best_ty;
    h->cfg.orient_per_cta = best_opc;
    if (tile_y) *tile_y = best_ty;
    if (opc) *opc = best_opc;
    if (us_per_pattern) *us_per_pattern = best_us;
    return EBSD_OK;
}

namespace {

// One launch of the pattern kernel's diagnostic instantiation: patterns
// into dout and the Lambert cells of every (orientation, pixel) into the
// four device arrays, all on the handle's stream.
int forward_cells_device(ebsd_handle* h, FwdParams p, const float4* dq, int64_t n, float* dout,
                         int32_t* nix, int32_t* niy, float* ixy0, float* ixy1)
{
    p.quats = dq;
    p.n = n;
    p.out = dout;
    p.nix = nix;
    p.niy = niy;
    p.ixy0 = ixy0;
    p.ixy1 = ixy1;
    cudaError_t e = launch_forward(p, h->NV, h->cfg, h->stream, true);
    if (e != cudaSuccess) return cuda_err(h, e, "pattern kernel (cells) launch");
    return EBSD_OK;
}

}  // namespace

extern "C" int ebsd_forward_cells(ebsd_handle* h, const float* quats, int64_t n,
                                  const ebsd_epilogue* e, float* out, int32_t* nix, int32_t* niy,
                                  float* ixy0, float* ixy1)
{
    int rc = check_ready(h);
    if (rc) return rc;
    if (n < 0 || !quats || !e || !out || !nix || !niy || !ixy0 || !ixy1)
        return set_err(h, EBSD_EINVAL, "ebsd_forward_cells: invalid arguments");
    if (n == 0) return EBSD_OK;
    if (e->poisson)
        return set_err(h, EBSD_EUNSUPPORTED, "ebsd_forward_cells: no noise in the cells variant");
    if (h->lambert_accurate == 2)
        return set_err(h, EBSD_EUNSUPPORTED,
                       "ebsd_forward_cells: no cells variant of the binary64 geometry");
    if (ptr_kind(quats) != kDevice || ptr_kind(out) != kDevice || ptr_kind(nix) != kDevice ||
        ptr_kind(niy) != kDevice || ptr_kind(ixy0) != kDevice || ptr_kind(ixy1) != kDevice)
        return set_err(h, EBSD_EINVAL, "ebsd_forward_cells: every array must be device memory");
    rc = check_device_home(h, "ebsd_forward_cells", {quats, out, nix, niy, ixy0, ixy1});
    if (rc) return rc;
    rc = check_aligned(h, quats, 16, "ebsd_forward_cells quats");
    if (rc) return rc;
    rc = activate(h);
    if (rc) return rc;
    FwdParams p;
    rc = fill_params(h, e, p);
    if (rc) return rc;
    return forward_cells_device(h, p, (const float4*)quats, n, out, nix, niy, ixy0, ixy1);
}

extern "C" int ebsd_cells(ebsd_handle* h, const float* quats, int64_t n, int32_t* nix,
                          int32_t* niy, float* ixy0, float* ixy1)
{
    int rc = check_ready(h);
    if (rc) return rc;
    if (n < 0 || !quats || !nix || !niy || !ixy0 || !ixy1)
        return set_err(h, EBSD_EINVAL, "ebsd_cells: invalid arguments");
    if (n == 0) return EBSD_OK;
    rc = check_device_home(h, "ebsd_cells", {quats, nix, niy, ixy0, ixy1});
    if (rc) return rc;
    if (h->lambert_accurate == 2)
        return set_err(h, EBSD_EUNSUPPORTED, "ebsd_cells: no cells variant of the binary64 geometry");
    rc = activate(h);
    if (rc) return rc;
    ebsd_epilogue unit;
    memset(&unit, 0, sizeof unit);
    unit.prefactor = 1.0;
    unit.binning = 1;
    unit.scalingmode = EBSD_SCALING_NOT;
    FwdParams p;
    rc = fill_params(h, &unit, p);
    if (rc) return rc;
    const size_t total = (size_t)n * h->P;
    const bool dev = ptr_kind(nix) == kDevice && ptr_kind(niy) == kDevice &&
                     ptr_kind(ixy0) == kDevice && ptr_kind(ixy1) == kDevice;
    cudaStream_t s = h->stream;
    // call-local buffers: quaternions (host input), the patterns the
    // kernel also writes, and the cells when the caller's are on the host
    DeviceBuf qb, ob;
    const float4* dq = (const float4*)quats;
    const bool qdev = ptr_kind(quats) == kDevice;
    if (qdev) {
        rc = check_aligned(h, quats, 16, "ebsd_cells quats");
        if (rc) return rc;
    } else {
        rc = check_quats_host(h, quats, n);
        if (rc) return rc;
    }
    const size_t qbytes = qdev ? 0 : ((sizeof(float4) * n + 255) & ~size_t(255));
    const size_t pbytes = (total * 4 + 255) & ~size_t(255);
    rc = ensure(h, ob, qbytes + pbytes + (dev ? 0 : total * 16), "cells staging");
    if (rc) return rc;
    char* base = (char*)ob.ptr;
    if (!qdev) {
        dq = (const float4*)base;
        cudaError_t ce =
            cudaMemcpyAsync(base, quats, sizeof(float4) * n, cudaMemcpyHostToDevice, s);
        if (ce != cudaSuccess) {
            cudaFree(ob.ptr);
            return cuda_err(h, ce, "ebsd_cells upload");
        }
    }
    float* dpat = (float*)(base + qbytes);
    int32_t *dnix = nix, *dniy = niy;
    float *d0 = ixy0, *d1 = ixy1;
    if (!dev) {
        char* c = base + qbytes + pbytes;
        dnix = (int32_t*)c;
        dniy = (int32_t*)(c + total * 4);
        d0 = (float*)(c + total * 8);
        d1 = (float*)(c + total * 12);
    }
    rc = forward_cells_device(h, p, dq, n, dpat, dnix, dniy, d0, d1);
    cudaError_t e = cudaSuccess;
    if (!rc && !dev) {
        e = cudaMemcpyAsync(nix, dnix, total * 4, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaMemcpyAsync(niy, dniy, total * 4, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaMemcpyAsync(ixy0, d0, total * 4, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaMemcpyAsync(ixy1, d1, total * 4, cudaMemcpyDeviceToHost, s);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cudaFree(ob.ptr);
    if (rc) return rc;
    if (e != cudaSuccess) return cuda_err(h, e, "ebsd_cells");
    return EBSD_OK;
}

extern "C" int ebsd_get_detector(ebsd_handle* h, float* W, float* rgx, float* rgy, float* rgz)
{
    int rc = check_ready(h);
    if (rc) return rc;
    rc = activate(h);
    if (rc) return rc;
    const int P = h->P;
    CK(h, cudaStreamSynchronize(h->stream), "sync");
    if (rgx || rgy || rgz) {
        std::vector<float4> rg(P);
        CK(h, cudaMemcpy(rg.data(), h->d_rg, sizeof(float4) * P, cudaMemcpyDeviceToHost), "rg");
        for (int i = 0; i < P; ++i) {
            if (rgx) rgx[i] = rg[i].x;
            if (rgy) rgy[i] = rg[i].y;
            if (rgz) rgz[i] = rg[i].z;
        }
    }
    if (W) {
        std::vector<float4> w((size_t)P * h->NV);
        CK(h, cudaMemcpy(w.data(), h->d_W, sizeof(float4) * w.size(), cudaMemcpyDeviceToHost), "W");
        const int nE = h->nE;
        memset(W, 0, sizeof(float) * (size_t)nE * P);
        const float* wf = (const float*)w.data();
        for (int p = 0; p < P; ++p)
            for (int k = 0; k < h->nsel; ++k) {
                const int c = k / 4, t = k % 4;
                W[(size_t)p * nE + (h->Emin - 1 + k)] = wf[((size_t)c * P + p) * 4 + t];
            }
    }
    return EBSD_OK;
}

// Internal accessors for the program driver (ebsd_program.cpp).
namespace ebsd {
namespace host {
float handle_max_sr(const ebsd_handle* h) { return h->ms ? h->ms->max_sr : 0.0f; }
int handle_set_error(ebsd_handle* h, int code, const char* msg)
{
    return set_err(h, code, "%s", msg);
}
int global_set_error(int code, const char* msg) { return set_err(nullptr, code, "%s", msg); }
}  // namespace host
}  // namespace ebsd

// ----------------------------------------------------------------------
// Orientation lists for dictionaries: cubochoric sampling of a Rodrigues
// fundamental zone (so3.f90:267-371)

namespace {

// so3.f90:73-74: FZ type and principal-axis order per point group 1..32
const int kFZtype[32] = {0, 0, 1, 1, 1, 2, 2, 2, 1, 1, 1, 2, 2, 2, 2, 1,
                         1, 2, 2, 2, 1, 1, 1, 2, 2, 2, 2, 3, 3, 4, 3, 4};
const int kFZorder[32] = {0, 0, 2, 2, 2, 2, 2, 2, 4, 4, 4, 4, 4, 4, 4, 3,
                          3, 3, 3, 3, 6, 6, 6, 6, 6, 6, 6, 0, 0, 0, 0, 0};

size_t align256(size_t b) { return (b + 255) & ~size_t(255); }

}  // namespace

extern "C" int ebsd_sample_rfz(ebsd_handle* h, int32_t nsteps, int32_t pgnum, double* rods,
                               float* quats, int64_t capacity, int64_t* count)
{
    if (!h) return set_err(nullptr, EBSD_EINVAL, "null handle");
    if (!count) return set_err(h, EBSD_EINVAL, "ebsd_sample_rfz: count is null");
    if (nsteps < 1 || nsteps > kMaxRfzSteps)
        return set_err(h, EBSD_EINVAL, "ebsd_sample_rfz: nsteps %d outside 1..%d", nsteps,
                       kMaxRfzSteps);
    if (pgnum < 1 || pgnum > 32)
        return set_err(h, EBSD_EINVAL, "ebsd_sample_rfz: point group %d outside 1..32", pgnum);
    if (capacity < 0) return set_err(h, EBSD_EINVAL, "ebsd_sample_rfz: negative capacity");
    int rc = activate(h);
    if (rc) return rc;
    const So3Consts K = so3_constants();
    // the grid coordinates exactly as the reference accumulates them
    std::vector<double> xs;
    const double delta = K.semi / (double)nsteps;
    for (double x = -K.semi; x < K.semi; x = x + delta) xs.push_back(x);
    const int m = (int)xs.size();
    const long long total = (long long)m * m * m;
    const long long nchunks = rfz_chunks(total);
    const size_t o_xs = 0, o_code = align256(sizeof(double) * m);
    const size_t o_chunk = o_code + align256((size_t)total);
    const size_t o_enter = o_chunk + align256(rfz_chunk_bytes() * (size_t)nchunks);
    const size_t o_off = o_enter + align256(sizeof(int) * (size_t)nchunks);
    const size_t o_cnt = o_off + align256(sizeof(long long) * (size_t)nchunks);
    rc = ensure(h, h->rfz, o_cnt + 256, "fundamental-zone sampling");
    if (rc) return rc;
    char* base = (char*)h->rfz.ptr;
    cudaStream_t s = h->stream;
    const bool want = capacity > 0 && (rods || quats);
    const bool rdev = rods && ptr_kind(rods) == kDevice;
    const bool qdev = quats && ptr_kind(quats) == kDevice;
    rc = check_device_home(h, "ebsd_sample_rfz", {rods, quats});
    if (rc) return rc;
    if (rdev) {
        rc = check_aligned(h, rods, 8, "ebsd_sample_rfz rods");
        if (rc) return rc;
    }
    if (qdev) {
        rc = check_aligned(h, quats, 16, "ebsd_sample_rfz quats");
        if (rc) return rc;
    }
    double* d_rods = rdev ? rods : nullptr;
    float* d_quats = qdev ? quats : nullptr;
    if (want && ((rods && !rdev) || (quats && !qdev))) {
        const size_t rb = rods && !rdev ? align256(sizeof(double) * 3 * (size_t)capacity) : 0;
        const size_t qb = quats && !qdev ? sizeof(float) * 4 * (size_t)capacity : 0;
        rc = ensure(h, h->rfz_out, rb + qb, "fundamental-zone sampling output");
        if (rc) return rc;
        if (rods && !rdev) d_rods = (double*)h->rfz_out.ptr;
        if (quats && !qdev) d_quats = (float*)((char*)h->rfz_out.ptr + rb);
    }
    CK(h, cudaMemcpyAsync(base + o_xs, xs.data(), sizeof(double) * m, cudaMemcpyHostToDevice, s),
       "grid upload");
    CK(h, launch_rfz(K, (const double*)(base + o_xs), m, kFZtype[pgnum - 1], kFZorder[pgnum - 1],
                     (uint8_t*)(base + o_code), base + o_chunk, (int*)(base + o_enter),
                     (long long*)(base + o_off), (long long*)(base + o_cnt),
                     want ? capacity : 0, want ? d_rods : nullptr, want ? d_quats : nullptr,
                     !want, s),
       "fundamental-zone sampling");
    long long n = 0;
    CK(h, cudaMemcpyAsync(&n, base + o_cnt, sizeof n, cudaMemcpyDeviceToHost, s), "count copy");
    CK(h, cudaStreamSynchronize(s), "fundamental-zone sampling");
    const long long w = want ? std::min<long long>(n, capacity) : 0;
    if (w > 0 && rods && !rdev)
        CK(h, cudaMemcpy(rods, d_rods, sizeof(double) * 3 * (size_t)w, cudaMemcpyDeviceToHost),
           "rods copy");
    if (w > 0 && quats && !qdev)
        CK(h, cudaMemcpy(quats, d_quats, sizeof(float) * 4 * (size_t)w, cudaMemcpyDeviceToHost),
           "quaternion copy");
    *count = n;
    return EBSD_OK;
}

// ----------------------------------------------------------------------
// Monte-Carlo backscatter histograms (CTEMMC.f90:307-529)

extern "C" int ebsd_mc_dims(const ebsd_mc_params* p, int32_t* numEbins, int32_t* numzbins)
{
    if (!p || !numEbins || !numzbins) return set_err(nullptr, EBSD_EINVAL, "ebsd_mc_dims: null");
    const bool ok = std::isfinite(p->EkeV) && std::isfinite(p->Ehistmin) &&
                    p->Ebinsize > 0.0 && p->depthstep > 0.0 && p->depthmax >= 0.0 &&
                    p->EkeV > p->Ehistmin && p->numsx >= 3 && (p->numsx % 2) == 1 &&
                    p->numsx <= 20001 && (p->EkeV - p->Ehistmin) / p->Ebinsize < 1.0e5 &&
                    p->depthmax / p->depthstep < 1.0e5;
    if (!ok)
        return set_err(nullptr, EBSD_EINVAL,
                       "Monte-Carlo parameters: need EkeV > Ehistmin, Ebinsize > 0, depthstep > "
                       "0, odd numsx in 3..20001");
    *numEbins = (int32_t)((p->EkeV - p->Ehistmin) / p->Ebinsize) + 1;
    *numzbins = (int32_t)(p->depthmax / p->depthstep) + 1;
    return EBSD_OK;
}

extern "C" int ebsd_mc_run(ebsd_handle* h, const ebsd_mc_params* p, uint64_t seed,
                           int64_t first_electron, int64_t n_electrons, int32_t* accum_e,
                           int32_t* accum_z, int64_t* counted)
{
    if (!h) return set_err(nullptr, EBSD_EINVAL, "null handle");
    if (!p || !accum_e) return set_err(h, EBSD_EINVAL, "ebsd_mc_run: null argument");
    int32_t nE = 0, nz = 0;
    if (ebsd_mc_dims(p, &nE, &nz) != EBSD_OK) return set_err(h, EBSD_EINVAL, "%s", g_err.c_str());
    if (!(p->Ze > 0.0) || !(p->density > 0.0) || !(p->at_wt > 0.0) || !std::isfinite(p->sig) ||
        !std::isfinite(p->omega) || std::fabs(p->omega) >= 90.0)
        return set_err(h, EBSD_EINVAL, "ebsd_mc_run: Ze, density, at_wt must be > 0, tilts finite");
    if (n_electrons < 0 || first_electron < 0)
        return set_err(h, EBSD_EINVAL, "ebsd_mc_run: negative electron range");
    int rc = activate(h);
    if (rc) return rc;
    const McConsts K = mc_constants(*p);
    const size_t ne = (size_t)nE * p->numsx * p->numsx;
    const size_t w10 = 2 * (size_t)K.nz10 + 1;
    const size_t nzs = (size_t)nE * nz * w10 * w10;
    const bool edev = ptr_kind(accum_e) == kDevice;
    const bool zdev = accum_z ? ptr_kind(accum_z) == kDevice : true;
    rc = check_device_home(h, "ebsd_mc_run", {accum_e, accum_z});
    if (rc) return rc;
    const size_t o_cnt = 0, o_e = 256;
    const size_t o_z = o_e + (edev ? 0 : ((ne * 4 + 255) & ~size_t(255)));
    rc = ensure(h, h->mc, o_z + (zdev ? 0 : nzs * 4) + 256, "Monte-Carlo histograms");
    if (rc) return rc;
    char* base = (char*)h->mc.ptr;
    int32_t* de = edev ? accum_e : (int32_t*)(base + o_e);
    int32_t* dz = accum_z ? (zdev ? accum_z : (int32_t*)(base + o_z)) : nullptr;
    unsigned long long* dcnt = (unsigned long long*)(base + o_cnt);
    cudaStream_t s = h->stream;
    CK(h, cudaMemsetAsync(de, 0, ne * 4, s), "histogram clear");
    if (dz) CK(h, cudaMemsetAsync(dz, 0, nzs * 4, s), "histogram clear");
    CK(h, cudaMemsetAsync(dcnt, 0, sizeof(unsigned long long), s), "counter clear");
    CK(h, launch_mc(K, seed, first_electron, n_electrons, de, dz, dcnt, h->mc_fp32 != 0, s),
       "Monte-Carlo kernel");
    unsigned long long c = 0;
    CK(h, cudaMemcpyAsync(&c, dcnt, sizeof c, cudaMemcpyDeviceToHost, s), "counter copy");
    if (!edev) CK(h, cudaMemcpyAsync(accum_e, de, ne * 4, cudaMemcpyDeviceToHost, s), "accum_e copy");
    if (accum_z && !zdev)
        CK(h, cudaMemcpyAsync(accum_z, dz, nzs * 4, cudaMemcpyDeviceToHost, s), "accum_z copy");
    CK(h, cudaStreamSynchronize(s), "Monte-Carlo");
    if (counted) *counted = (int64_t)c;
    return EBSD_OK;
}

// ----------------------------------------------------------------------
// Roofline denominators

extern "C" int ebsd_measure_bandwidth(int32_t device, int32_t level, int64_t bytes,
                                      int32_t repeats, double* gbs)
{
    if (!gbs) return set_err(nullptr, EBSD_EINVAL, "ebsd_measure_bandwidth: null output");
    if (level != EBSD_BW_L1 && level != EBSD_BW_L2 && level != EBSD_BW_HBM)
        return set_err(nullptr, EBSD_EINVAL, "ebsd_measure_bandwidth: unknown level %d", level);
    if (bytes < 16 || bytes > (int64_t(64) << 30) || repeats < 1 || repeats > 1000)
        return set_err(nullptr, EBSD_EINVAL,
                       "ebsd_measure_bandwidth: bytes in 16 B..64 GiB, repeats in 1..1000");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) {
        cudaGetLastError();
        return set_err(nullptr, EBSD_EINVAL, "ebsd_measure_bandwidth: no device %d", device);
    }
    int prev = 0;
    cudaGetDevice(&prev);
    cudaError_t e = measure_read_bandwidth(device, level, bytes, repeats, gbs, nullptr);
    cudaSetDevice(prev);
    if (e != cudaSuccess) return cuda_err(nullptr, e, "ebsd_measure_bandwidth");
    return EBSD_OK;
}
