// Orientation lists for EBSD dictionaries: cubochoric sampling of a
// Rodrigues fundamental zone (SampleRFZ, so3.f90:267-371), in binary64 as
// the reference, producing the Rodrigues vectors and the float32
// quaternions ebsd_forward consumes.
//
// The reference walks the (2N+1)^3 grid sequentially and keeps a flag that
// FZ types 0 and 1 leave untouched for rotations of 179.999 degrees and
// more, so a point's membership can depend on the points before it.  The
// GPU version splits the walk into three passes:
//   1. k_rfz_code   one thread per grid point: cube -> ball -> Rodrigues
//                   vector and the FZ test, a code 0/1 (assigned) or 2
//                   (keeps the previous value);
//   2. k_rfz_chunks one warp per 1024 points: a scan of the codes under the
//                   associative composition of (assigned?, last value,
//                   count if entering false, count if entering true);
//   3. k_rfz_prefix one block: the same composition over the chunks gives
//                   each chunk its entering value and output offset;
//   4. k_rfz_write  one warp per chunk again: each lane walks its 32 points
//                   and writes the members in grid order.
#include <algorithm>
#include <cmath>
#include <cstdint>

#include "ebsd_internal.h"

namespace ebsd {

namespace {

constexpr int kRfzLanePts = 32;                       // points per lane
constexpr int kRfzChunk = 32 * kRfzLanePts;           // points per warp

// Homochoric -> angle fit, rotations.f90:2596-2599.
__constant__ double c_tfit[7] = {-0.5000096149170321, -0.02486606148871731,
                                 -0.004549381779362819, 0.0005118668366387526,
                                 -0.0016500827333575548, 0.0007593352203388718,
                                 -0.0002040422502566876};

__device__ __forceinline__ double maxabs3(double a, double b, double c)
{
    return fmax(fabs(a), fmax(fabs(b), fabs(c)));
}

// Lambert.f90:1314-1365 (0: no pyramid, NaN input)
__device__ __forceinline__ int pyramid(double x, double y, double z)
{
    if (fabs(x) <= z && fabs(y) <= z) return 1;
    if (fabs(x) <= -z && fabs(y) <= -z) return 2;
    if (fabs(z) <= x && fabs(y) <= x) return 3;
    if (fabs(z) <= -x && fabs(y) <= -x) return 4;
    if (fabs(x) <= y && fabs(z) <= y) return 5;
    if (fabs(x) <= -y && fabs(z) <= -y) return 6;
    return 0;
}

// Cubochoric -> homochoric (Lambert.f90:960-1030), then -> Rodrigues
// (rotations.f90:2584-2619).
__device__ void cu2ro(const So3Consts& K, double cx, double cy, double cz, double r[3])
{
    r[0] = r[1] = r[2] = 0.0;
    if (maxabs3(cx, cy, cz) > K.edge) return;
    const int p = pyramid(cx, cy, cz);
    double s0 = cx, s1 = cy, s2 = cz;
    if (p == 3 || p == 4) {
        s0 = cy; s1 = cz; s2 = cx;
    } else if (p == 5 || p == 6) {
        s0 = cz; s1 = cx; s2 = cy;
    }
    const double X0 = K.sc * s0, X1 = K.sc * s1, X2 = K.sc * s2;
    double l0 = 0.0, l1 = 0.0, l2 = 0.0;
    if (maxabs3(X0, X1, X2) == 0.0) {
    } else if (fmax(fabs(X0), fabs(X1)) == 0.0) {
        l2 = K.pref * X2;
    } else {
        double cc, ss, q, T1, T2;
        if (fabs(X1) <= fabs(X0)) {
            const double t = K.pi12 * X1 / X0;
            cc = cos(t);
            ss = sin(t);
            q = K.prek * X0 / sqrt(K.r2 - cc);
            T1 = (K.r2 * cc - 1.0) * q;
            T2 = K.r2 * ss * q;
        } else {
            const double t = K.pi12 * X0 / X1;
            cc = cos(t);
            ss = sin(t);
            q = K.prek * X1 / sqrt(K.r2 - cc);
            T1 = K.r2 * ss * q;
            T2 = (K.r2 * cc - 1.0) * q;
        }
        cc = T1 * T1 + T2 * T2;
        ss = K.Pi * cc / (24.0 * (X2 * X2));
        cc = K.sPi * cc / K.r24 / X2;
        q = sqrt(1.0 - ss);
        l0 = T1 * q;
        l1 = T2 * q;
        l2 = K.pref * X2 - cc;
    }
    double h0 = l0, h1 = l1, h2 = l2;
    if (p == 3 || p == 4) {
        h0 = l2; h1 = l0; h2 = l1;
    } else if (p == 5 || p == 6) {
        h0 = l1; h1 = l2; h2 = l0;
    }
    const double hmag = h0 * h0 + h1 * h1 + h2 * h2;
    if (hmag == 0.0) return;
    const double sq = sqrt(hmag);
    double hm = hmag, s = c_tfit[0] * hmag;
#pragma unroll
    for (int i = 1; i < 7; ++i) {
        hm = hm * hmag;
        s = s + c_tfit[i] * hm;
    }
    s = tan(acos(1.0 + s));
    r[0] = h0 / sq * s;
    r[1] = h1 / sq * s;
    r[2] = h2 / sq * s;
}

// so3.f90:105-245 with the loop's use of the result (:326-340): 1/0 when
// the body assigns insideFZ, 2 when it keeps the previous value.
__device__ int fz_code(const So3Consts& K, int type, int order, const double r[3])
{
    const double rx = r[0], ry = r[1], rz = r[2];
    switch (type) {
        case 0: return rx * rx + ry * ry + rz * rz < K.rvmax2 ? 1 : 2;
        case 1:
            if (!(rx * rx + ry * ry + rz * rz < K.rvmax2)) return 2;
            return fabs(rz) <= K.BP[order - 1] ? 1 : 0;
        case 2: {
            if (!(fabs(rz) <= K.BP[order - 1])) return 0;
            bool c2 = false;
            if (order == 2 || order == 4) {
                c2 = fabs(rx) <= 1.0 && fabs(ry) <= 1.0;
                if (order == 4)
                    c2 = c2 && (K.r22 * fabs(rx + ry) <= 1.0 && K.r22 * fabs(rx - ry) <= 1.0);
            } else if (order == 3) {
                c2 = fabs(K.srt * rx + 0.5 * ry) <= 1.0 && fabs(K.srt * rx - 0.5 * ry) <= 1.0 &&
                     fabs(ry) <= 1.0;
            } else if (order == 6) {
                c2 = fabs(0.5 * rx + K.srt * ry) <= 1.0 && fabs(K.srt * rx + 0.5 * ry) <= 1.0 &&
                     fabs(K.srt * rx - 0.5 * ry) <= 1.0 && fabs(0.5 * rx - K.srt * ry) <= 1.0 &&
                     fabs(ry) <= 1.0 && fabs(rx) <= 1.0;
            }
            return c2 ? 1 : 0;
        }
        default: {
            const bool c1 = type == 3 || maxabs3(rx, ry, rz) <= K.pi8;
            const bool c2 = fabs(rx + ry + rz) <= 1.0 && fabs(-rx + ry + rz) <= 1.0 &&
                            fabs(rx - ry + rz) <= 1.0 && fabs(rx + ry - rz) <= 1.0;
            return (c1 && c2) ? 1 : 0;
        }
    }
}

// ro2qu_d = om2qu_d(ax2om_d(ro2ax_d(r))) (rotations.f90:2233-2242,
// 1209-1229, 791-824, 1618-1647); a zero vector gives the identity.
__device__ void ro2qu(const double r[3], double q[4])
{
    double ta = sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
    if (ta == 0.0) {
        q[0] = 1.0;
        q[1] = q[2] = q[3] = 0.0;
        return;
    }
    const double angle = 2.0 * atan(ta);
    double a0 = r[0] / ta, a1 = r[1] / ta, a2 = r[2] / ta;
    ta = sqrt(a0 * a0 + a1 * a1 + a2 * a2);
    a0 = a0 / ta;
    a1 = a1 / ta;
    a2 = a2 / ta;
    const double c = cos(angle), s = sin(angle), omc = 1.0 - c;
    const double m00 = a0 * a0 * omc + c, m11 = a1 * a1 * omc + c, m22 = a2 * a2 * omc + c;
    double t = omc * a0 * a1;
    const double m01 = t + s * a2, m10 = t - s * a2;
    t = omc * a1 * a2;
    const double m12 = t + s * a0, m21 = t - s * a0;
    t = omc * a2 * a0;
    const double m20 = t + s * a1, m02 = t - s * a1;
    q[0] = sqrt(fabs(m00 + m11 + m22 + 1.0)) / 2.0;
    q[1] = sqrt(fabs(m00 - m11 - m22 + 1.0)) / 2.0;
    q[2] = sqrt(fabs(-m00 + m11 - m22 + 1.0)) / 2.0;
    q[3] = sqrt(fabs(-m00 - m11 + m22 + 1.0)) / 2.0;
    if (m21 - m12 < 0.0) q[1] = -q[1];
    if (m02 - m20 < 0.0) q[2] = -q[2];
    if (m10 - m01 < 0.0) q[3] = -q[3];
    const double n = 1.0 / sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3]);
    for (int i = 0; i < 4; ++i) q[i] = n * q[i];
}

struct Walk {  // summary of a run of codes
    int has;   // some point assigned the flag
    int last;  // the value after the run (when has)
    long long cf, ct;  // members when the run is entered with false / true
};

__device__ __forceinline__ Walk compose(const Walk& a, const Walk& b)
{
    Walk r;
    r.has = a.has | b.has;
    r.last = b.has ? b.last : a.last;
    const long long bf = a.has ? (a.last ? b.ct : b.cf) : b.cf;
    const long long bt = a.has ? (a.last ? b.ct : b.cf) : b.ct;
    r.cf = a.cf + bf;
    r.ct = a.ct + bt;
    return r;
}

__device__ __forceinline__ Walk walk_points(const uint8_t* code, long long i0, long long total)
{
    Walk w = {0, 0, 0, 0};
    for (int k = 0; k < kRfzLanePts; ++k) {
        const long long i = i0 + k;
        if (i >= total) break;
        const int c = code[i];
        if (c == 2) {
            w.cf += w.has ? w.last : 0;
            w.ct += w.has ? w.last : 1;
        } else {
            w.has = 1;
            w.last = c;
            w.cf += c;
            w.ct += c;
        }
    }
    return w;
}

// inclusive warp scan of lane summaries
__device__ __forceinline__ Walk warp_scan(Walk w, int lane)
{
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        Walk o;
        o.has = __shfl_up_sync(0xffffffffu, w.has, off);
        o.last = __shfl_up_sync(0xffffffffu, w.last, off);
        o.cf = __shfl_up_sync(0xffffffffu, w.cf, off);
        o.ct = __shfl_up_sync(0xffffffffu, w.ct, off);
        if (lane >= off) w = compose(o, w);
    }
    return w;
}

__global__ void k_rfz_code(const So3Consts K, const double* __restrict__ xs, int m, int type,
                           int order, uint8_t* __restrict__ code)
{
    const long long total = (long long)m * m * m;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const int ix = (int)(i / ((long long)m * m));
        const int iy = (int)((i / m) % m);
        const int iz = (int)(i % m);
        double r[3];
        cu2ro(K, xs[ix], xs[iy], xs[iz], r);
        code[i] = (uint8_t)fz_code(K, type, order, r);
    }
}

__global__ void k_rfz_chunks(const uint8_t* __restrict__ code, long long total, long long nchunks,
                             Walk* __restrict__ chunk)
{
    const long long c = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (c >= nchunks) return;  // whole warps leave together
    Walk w = walk_points(code, c * kRfzChunk + (long long)lane * kRfzLanePts, total);
    w = warp_scan(w, lane);
    if (lane == 31) chunk[c] = w;
}

// One block: chunk summaries -> entering value and offset per chunk.
__global__ void k_rfz_prefix(const Walk* __restrict__ chunk, long long nchunks,
                             int* __restrict__ enter, long long* __restrict__ offset,
                             long long* __restrict__ count)
{
    __shared__ Walk sh[1024];
    const int t = threadIdx.x, nt = blockDim.x;
    const long long per = (nchunks + nt - 1) / nt;
    const long long c0 = t * per, c1 = min(nchunks, c0 + per);
    Walk w = {0, 0, 0, 0};
    for (long long c = c0; c < c1; ++c) w = compose(w, chunk[c]);
    sh[t] = w;
    __syncthreads();
    for (int off = 1; off < nt; off <<= 1) {  // Hillis-Steele inclusive scan
        Walk o = sh[t];
        if (t >= off) o = compose(sh[t - off], o);
        __syncthreads();
        sh[t] = o;
        __syncthreads();
    }
    Walk pre = t > 0 ? sh[t - 1] : Walk{0, 0, 0, 0};  // exclusive prefix
    for (long long c = c0; c < c1; ++c) {
        const int v = pre.has ? pre.last : 0;  // the flag starts false
        enter[c] = v;
        offset[c] = pre.cf;
        pre = compose(pre, chunk[c]);
    }
    if (t == nt - 1) *count = sh[nt - 1].cf;
}

__global__ void k_rfz_write(const So3Consts K, const double* __restrict__ xs, int m,
                            const uint8_t* __restrict__ code, long long total, long long nchunks,
                            const int* __restrict__ enter, const long long* __restrict__ offset,
                            long long cap, double* __restrict__ rods, float* __restrict__ quats)
{
    const long long c = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (c >= nchunks) return;
    const long long i0 = c * kRfzChunk + (long long)lane * kRfzLanePts;
    const Walk own = walk_points(code, i0, total);
    const Walk inc = warp_scan(own, lane);
    Walk ex;
    ex.has = __shfl_up_sync(0xffffffffu, inc.has, 1);
    ex.last = __shfl_up_sync(0xffffffffu, inc.last, 1);
    ex.cf = __shfl_up_sync(0xffffffffu, inc.cf, 1);
    ex.ct = __shfl_up_sync(0xffffffffu, inc.ct, 1);
    if (lane == 0) ex = Walk{0, 0, 0, 0};
    const int e = enter[c];
    int flag = ex.has ? ex.last : e;
    long long pos = offset[c] + (e ? ex.ct : ex.cf);
    for (int k = 0; k < kRfzLanePts; ++k) {
        const long long i = i0 + k;
        if (i >= total) break;
        const int cd = code[i];
        if (cd != 2) flag = cd;
        if (!flag) continue;
        if (pos < cap) {
            const int ix = (int)(i / ((long long)m * m));
            const int iy = (int)((i / m) % m);
            const int iz = (int)(i % m);
            double r[3];
            cu2ro(K, xs[ix], xs[iy], xs[iz], r);
            if (rods) {
                rods[3 * pos] = r[0];
                rods[3 * pos + 1] = r[1];
                rods[3 * pos + 2] = r[2];
            }
            if (quats) {
                double q[4];
                ro2qu(r, q);
                reinterpret_cast<float4*>(quats)[pos] =
                    make_float4((float)q[0], (float)q[1], (float)q[2], (float)q[3]);
            }
        }
        ++pos;
    }
}

}  // namespace

// Lambert.f90:246-280, evaluated on the host with the C library.
So3Consts so3_constants()
{
    So3Consts K;
    const double dpi = 4.0 * std::atan(1.0);
    K.Pi = dpi;
    K.sPi = std::sqrt(dpi);
    K.srt = std::sqrt(3.0) / 2.0;
    K.pref = std::sqrt(6.0 / dpi);
    const double a = std::pow(dpi, 5.0 / 6.0) / std::pow(6.0, 1.0 / 6.0);
    const double ap = std::pow(dpi, 2.0 / 3.0);
    K.semi = 0.5 * ap;
    K.sc = a / ap;
    const double beta = 0.5 * a;
    K.R1 = std::pow(3.0 * dpi / 4.0, 1.0 / 3.0);
    K.r2 = std::sqrt(2.0);
    K.r22 = std::sqrt(2.0) / 2.0;
    K.pi12 = dpi / 12.0;
    K.pi8 = std::tan(dpi / 8.0);
    K.prek = K.R1 * std::pow(2.0, 0.25) / beta;
    K.r24 = std::sqrt(24.0);
    const double t = std::tan(179.999 * dpi / 2.0 / 180.0);
    K.rvmax2 = t * t;
    K.BP[0] = 0.0;
    K.BP[1] = std::tan(dpi / 4.0);
    K.BP[2] = std::tan(dpi / 6.0);
    K.BP[3] = K.pi8;
    K.BP[4] = 0.0;
    K.BP[5] = std::tan(K.pi12);
    K.edge = 0.5 * std::pow(3.141592653589793238, 2.0 / 3.0);
    return K;
}

long long rfz_chunks(long long total) { return (total + kRfzChunk - 1) / kRfzChunk; }

size_t rfz_chunk_bytes() { return sizeof(Walk); }

cudaError_t launch_rfz(const So3Consts& K, const double* xs, int m, int type, int order,
                       uint8_t* code, void* chunk, int* enter, long long* offset,
                       long long* count, long long cap, double* rods, float* quats,
                       bool count_only, cudaStream_t s)
{
    const long long total = (long long)m * m * m;
    const long long nchunks = rfz_chunks(total);
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const long long want = (total + 255) / 256;
    const int g1 = (int)std::min<long long>(want, (long long)sms * 16);
    k_rfz_code<<<g1, 256, 0, s>>>(K, xs, m, type, order, code);
    const unsigned g2 = (unsigned)((nchunks * 32 + 255) / 256);
    k_rfz_chunks<<<g2, 256, 0, s>>>(code, total, nchunks, (Walk*)chunk);
    k_rfz_prefix<<<1, 1024, 0, s>>>((const Walk*)chunk, nchunks, enter, offset, count);
    if (!count_only)
        k_rfz_write<<<g2, 256, 0, s>>>(K, xs, m, code, total, nchunks, enter, offset, cap, rods,
                                       quats);
    return cudaGetLastError();
}

}  // namespace ebsd
