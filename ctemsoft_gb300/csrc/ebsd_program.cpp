// The CTEMEBSD program on the GPU: CTEMEBSD.f90:87-672 end to end, with the
// pattern loop replaced by libebsdgpu calls and the output written by a
// writer thread while the next chunk of patterns is computed.  On several
// GPUs the orientation loop (:573) is split into contiguous shards, one per
// device and host thread, and every shard writes its records at their own
// offsets in the one output file (:654-658).
#include <cuda_runtime.h>
#include <fcntl.h>
#include <unistd.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <string>
#include <thread>
#include <vector>

#include "ebsd_host.h"

using namespace ebsd;

namespace {

struct HandleGuard {
    ebsd_handle* h = nullptr;
    ~HandleGuard() { ebsd_destroy(h); }
};

struct PinnedGuard {
    float* p[2] = {nullptr, nullptr};
    ~PinnedGuard()
    {
        for (auto q : p)
            if (q) cudaFreeHost(q);
    }
};

int fail(int code, const std::string& msg)
{
    host::global_set_error(code, msg.c_str());
    return code;
}

}  // namespace

namespace {

// Positional writer of the output file: the header record, then one
// gfortran sequential record per pattern at the offset its index gives, so
// that shards on several GPUs write their records concurrently (pwrite on
// one descriptor) and the file equals the sequential one byte for byte.
class RecordFile {
public:
    static constexpr size_t kMaxSub = 2147483639u;  // gfortran's largest sub-record

    RecordFile(const char* path, size_t rec_bytes, long long keep_records)
        : rec_(rec_bytes)
    {
        const size_t nsub = rec_bytes == 0 ? 1 : (rec_bytes + kMaxSub - 1) / kMaxSub;
        per_ = (long long)rec_bytes + 8LL * (long long)nsub;
        if (keep_records > 0) {
            fd_ = ::open(path, O_RDWR);
            // drop whatever follows the kept records (a partial or lone record)
            if (fd_ >= 0 && ::ftruncate(fd_, (off_t)(20 + keep_records * per_)) != 0) {
                ::close(fd_);
                fd_ = -1;
            }
        } else {
            fd_ = ::open(path, O_RDWR | O_CREAT | O_TRUNC, 0644);
        }
    }
    ~RecordFile() { close(); }
    bool ok() const { return fd_ >= 0; }
    bool write_header(const int32_t hdr[3])
    {
        const int32_t m = 12;
        return put(0, &m, 4) && put(4, hdr, 12) && put(16, &m, 4);
    }
    // record k (0-based pattern index) from rec_ bytes at data
    bool write_record(long long k, const void* data)
    {
        long long off = 20 + k * per_;
        const char* p = (const char*)data;
        size_t left = rec_;
        bool first = true;
        do {
            const size_t n = left > kMaxSub ? kMaxSub : left;
            const bool more = left > n;
            const int32_t head = more ? -(int32_t)n : (int32_t)n;
            const int32_t tail = first ? (int32_t)n : -(int32_t)n;
            if (!put(off, &head, 4) || !put(off + 4, p, n) || !put(off + 4 + (long long)n, &tail, 4))
                return false;
            off += (long long)n + 8;
            p += n;
            left -= n;
            first = false;
        } while (left > 0);
        return true;
    }
    bool close()
    {
        if (fd_ < 0) return true;
        const bool ok = ::close(fd_) == 0;
        fd_ = -1;
        return ok;
    }

private:
    bool put(long long off, const void* data, size_t n)
    {
        const char* p = (const char*)data;
        while (n > 0) {
            const ssize_t w = ::pwrite(fd_, p, n, (off_t)off);
            if (w <= 0) return false;
            p += w;
            off += w;
            n -= (size_t)w;
        }
        return true;
    }
    int fd_ = -1;
    size_t rec_ = 0;
    long long per_ = 0;
};

// Complete records at the start of an existing output file with this
// header: every record's two length markers are checked, because shards
// written in parallel can leave a later record complete behind a missing
// one.
int64_t complete_records(const char* path, const int32_t hdr[3], size_t rec, int64_t numeuler)
{
    FILE* f = fopen(path, "rb");
    if (!f) return 0;
    int32_t head[5] = {0, 0, 0, 0, 0};
    int64_t done = 0;
    if (fread(head, 4, 5, f) == 5 && head[0] == 12 && head[4] == 12 && head[1] == hdr[0] &&
        head[2] == hdr[1] && head[3] == hdr[2]) {
        const long long per = 4LL * (long long)rec + 8;
        for (; done < numeuler; ++done) {
            const long long off = 20 + done * per;
            int32_t m1 = 0, m2 = 0;
            if (fseeko(f, (off_t)off, SEEK_SET) != 0 || fread(&m1, 4, 1, f) != 1 ||
                m1 != (int32_t)(4 * rec) ||
                fseeko(f, (off_t)(off + 4 + 4LL * (long long)rec), SEEK_SET) != 0 ||
                fread(&m2, 4, 1, f) != 1 || m2 != m1)
                break;
        }
    }
    fclose(f);
    return done;
}

// One GPU's shard [begin, end): patterns in chunks into a pinned double
// buffer, each chunk's records written by a writer thread while the next
// chunk is computed.
int run_shard(ebsd_handle* h, int device, const float* quats, int64_t begin, int64_t end,
              const ebsd_epilogue* epi, size_t rec, RecordFile* out, std::string* err)
{
    if (begin >= end) return EBSD_OK;
    if (cudaSetDevice(device) != cudaSuccess) {
        cudaGetLastError();
        *err = "cudaSetDevice failed";
        return EBSD_ECUDA;
    }
    const int64_t n = end - begin;
    const int64_t chunk = std::max<int64_t>(
        1, std::min<int64_t>(n, (int64_t)((size_t(256) << 20) / (rec * sizeof(float)))));
    PinnedGuard pg;
    for (int b = 0; b < 2; ++b) {
        if (cudaMallocHost(&pg.p[b], std::max<size_t>(1, chunk * rec) * sizeof(float)) !=
            cudaSuccess) {
            cudaGetLastError();
            *err = "pinned output buffer";
            return EBSD_ENOMEM;
        }
    }
    std::thread writer;
    std::atomic<bool> write_ok(true);
    int rc = EBSD_OK;
    // a chunk's records are written by up to kWriters threads, each a
    // contiguous run of them (positional writes at distinct offsets): one
    // thread copying into the page cache runs at ~4.5 GB/s, well below
    // what the device produces
    static constexpr int64_t kWriters = 4;
    auto write_chunk = [out, &write_ok, rec](const float* src, int64_t first, int64_t m) {
        const int64_t nt = std::min<int64_t>(kWriters, m);
        std::vector<std::thread> ws;
        for (int64_t w = 0; w < nt; ++w) {
            const int64_t a = m * w / nt, b = m * (w + 1) / nt;
            ws.emplace_back([out, &write_ok, src, first, a, b, rec] {
                for (int64_t k = a; k < b && write_ok.load(std::memory_order_relaxed); ++k)
                    if (!out->write_record(first + k, src + (size_t)k * rec))  // one record per pattern
                        write_ok = false;
            });
        }
        for (auto& t : ws) t.join();
    };
    for (int64_t o0 = begin, c = 0; o0 < end; o0 += chunk, ++c) {
        const int64_t m = std::min(chunk, end - o0);
        float* buf = pg.p[c & 1];
        // noise keyed by the pattern's index in the whole list, so that the
        // records do not depend on the chunk or shard that computes them
        rc = ebsd_set_option(h, "noise_index_offset", o0);
        if (!rc) rc = ebsd_forward(h, quats + 4 * o0, m, epi, buf);
        if (rc) {
            *err = ebsd_last_error(h);
            break;
        }
        if (writer.joinable()) writer.join();
        if (!write_ok) break;
        writer = std::thread([&write_chunk, buf, o0, m] { write_chunk(buf, o0, m); });
    }
    if (writer.joinable()) writer.join();
    if (rc) return rc;
    if (!write_ok) {
        *err = "output file write failed";
        return EBSD_EIO;
    }
    return EBSD_OK;
}

}  // namespace

extern "C" int ebsd_run_namelist(const char* nmlfile, int device, int quiet)
{
    const int32_t d = device;
    return ebsd_run_namelist_devices(nmlfile, &d, 1, quiet);
}

extern "C" int ebsd_run_namelist_devices(const char* nmlfile, const int32_t* devices,
                                         int32_t ndev, int quiet)
{
    auto say = [&](const char* fmt, auto... args) {
        if (!quiet) {
            printf(fmt, args...);
            fflush(stdout);
        }
    };
    if (!devices || ndev < 1 || ndev > 64)
        return fail(EBSD_EINVAL, "ebsd_run_namelist_devices: 1 to 64 devices");
    say(" CTEMEBSD (GB300): Dynamical EBSD patterns, using precomputed MC and master Lambert "
        "projections\n");

    ebsd_namelist nml;
    std::string err;
    int rc = host::read_namelist(nmlfile, &nml, &err);
    if (rc) return fail(rc, err);

    // angle file (:228-288), or a dictionary's fundamental-zone sampling
    // (the plan of :292-298), drawn once the device is set up
    std::vector<float> quats;
    int64_t numeuler = 0;
    const bool dictionary = nml.ncubochoric > 0;
    if (!dictionary) {
        rc = host::read_angle_file(nml.anglefile, nml.eulerconvention, nml.axisangle, &quats,
                                   &err);
        if (rc) return fail(rc, err);
        numeuler = (int64_t)(quats.size() / 4);
        say(" Number of angle entries = %lld\n", (long long)numeuler);
    }

    // MC file (:316-367)
    say(" opening %s\n", nml.energyfile);
    ebsd_mc_header mc;
    std::vector<int32_t> accum_e;
    rc = host::read_mc_file(nml.energyfile, &mc, &accum_e, nullptr, &err);
    if (rc) return fail(rc, err);
    say("  -> completed reading %s\n", nml.energyfile);
    const int nsx = (mc.numsx - 1) / 2, nsy = (mc.numsy - 1) / 2;
    int32_t Emin, Emax;
    host::energy_window(nml.energymin, nml.energymax, mc.Ehistmin, mc.Ebinsize, mc.numEbins, &Emin,
                        &Emax);
    int64_t mcsum = 0;
    for (int32_t v : accum_e) mcsum += v;
    say(" shape(accum_e) = %d %d %d\n", mc.numEbins, 2 * nsx + 1, 2 * nsy + 1);
    say(" energy range (Emin, Emax) = %d %d %lld\n", Emin, Emax, (long long)mcsum);

    // master file (:378-406)
    ebsd_master_header mh;
    std::vector<float> srtmp;
    rc = host::read_master_file(nml.FZfile, &mh, nullptr, nullptr, nullptr, &srtmp, &err);
    if (rc) return fail(rc, err);
    if (mh.nE != mc.numEbins) {
        char buf[256];
        snprintf(buf, sizeof buf,
                 "Energy histogram and Lambert stack have different energy dimension; aborting "
                 "program (histogram %d, Lambert stack %d)",
                 mc.numEbins, mh.nE);
        return fail(EBSD_EINVAL, buf);
    }
    say(" -> completed reading Master EBSD pattern file\n");

    // one handle per listed device (a device listed twice gets two handles
    // that share one device copy of the master and detector tables)
    std::vector<HandleGuard> hg(ndev);
    for (int k = 0; k < ndev; ++k) {
        rc = ebsd_create(&hg[k].h, devices[k]);
        if (rc) return rc;
    }
    ebsd_handle* h = hg[0].h;
    auto herr = [&](ebsd_handle* hh, int code) {
        host::global_set_error(code, ebsd_last_error(hh));
        return code;
    };
    if (dictionary) {
        int64_t cnt = 0;
        rc = ebsd_sample_rfz(h, nml.ncubochoric, nml.pgnum, nullptr, nullptr, 0, &cnt);
        if (rc) return herr(h, rc);
        quats.resize((size_t)cnt * 4);
        rc = ebsd_sample_rfz(h, nml.ncubochoric, nml.pgnum, nullptr, quats.data(), cnt, &cnt);
        if (rc) return herr(h, rc);
        host::apply_axisangle(nml.axisangle, quats.data(), cnt);
        numeuler = cnt;
        say(" Cubochoric sampling, %d steps, point group %d: %lld orientations in the "
            "fundamental zone\n", nml.ncubochoric, nml.pgnum, (long long)numeuler);
    }

    ebsd_geometry g;
    g.L = nml.L;
    g.thetac = nml.thetac;
    g.delta = nml.delta;
    g.numsx = nml.numsx;
    g.numsy = nml.numsy;
    g.xpc = nml.xpc;
    g.ypc = nml.ypc;
    g.sig = mc.sig;
    // set-up on every distinct device, concurrently
    std::vector<int> first(ndev);
    for (int k = 0; k < ndev; ++k) {
        first[k] = k;
        for (int j = 0; j < k; ++j)
            if (devices[j] == devices[k]) {
                first[k] = j;
                break;
            }
    }
    std::vector<int> src_rc(ndev, EBSD_OK);
    std::vector<int32_t> num_els(ndev, 0);
    {
        std::vector<std::thread> th;
        for (int k = 0; k < ndev; ++k) {
            if (first[k] != k) continue;
            th.emplace_back([&, k] {
                ebsd_handle* hk = hg[k].h;
                int r = ebsd_set_master(hk, srtmp.data(), mh.npx, mh.npy, mh.nE, mh.numset);
                if (!r)
                    r = ebsd_set_detector(hk, &g, accum_e.data(), nsx, nsy, mc.numEbins, Emin,
                                          Emax, &num_els[k]);
                src_rc[k] = r;
            });
        }
        for (auto& t : th) t.join();
    }
    for (int k = 0; k < ndev; ++k)
        if (first[k] == k && src_rc[k]) return herr(hg[k].h, src_rc[k]);
    for (int k = 0; k < ndev; ++k) {
        if (first[k] == k) continue;
        rc = ebsd_share_detector(hg[k].h, hg[first[k]].h);
        if (rc) return herr(hg[k].h, rc);
        num_els[k] = num_els[first[k]];
    }
    srtmp.clear();
    srtmp.shrink_to_fit();
    accum_e.clear();
    accum_e.shrink_to_fit();
    const int32_t num_el = num_els[0];
    for (int k = 1; k < ndev; ++k)
        if (num_els[k] != num_el)
            return fail(EBSD_ECUDA, "devices disagree on num_el");

    const double pref = host::prefactor(nml.beamcurrent, nml.dwelltime, num_el);
    {
        std::vector<float> W((size_t)mc.numEbins * g.numsx * g.numsy);
        rc = ebsd_get_detector(h, W.data(), nullptr, nullptr, nullptr);
        if (rc) return herr(h, rc);
        float wmax = W.empty() ? 0.0f : *std::max_element(W.begin(), W.end());
        say(" intensity prefactor = %.15g\n", pref);
        say(" max accum_e_detector = %.8g\n", wmax);
        say(" max sr = %.8g\n", host::handle_max_sr(h));
    }

    ebsd_epilogue epi;
    memset(&epi, 0, sizeof epi);
    epi.prefactor = pref;
    epi.binning = nml.binning;
    const std::string mode(nml.scalingmode);
    epi.scalingmode = mode == "not" ? EBSD_SCALING_NOT
                      : mode == "gam" ? EBSD_SCALING_GAM
                                      : EBSD_SCALING_LIN;  // any other value bins (:630)
    epi.gammavalue = nml.gammavalue;
    epi.poisson = nml.poisson;
    epi.seed = (uint64_t)nml.seed;
    int32_t rx = 0, ry = 0;
    rc = ebsd_output_dims(h, &epi, &rx, &ry);
    if (rc) return herr(h, rc);

    // output header (:555-561): binned dimensions whenever binning != 1
    int32_t hdr[3] = {nml.numsx, nml.numsy, (int32_t)numeuler};
    if (nml.binning != 1) {
        hdr[0] = nml.numsx / nml.binning;
        hdr[1] = nml.numsy / nml.binning;
    }
    const size_t rec = (size_t)rx * ry;
    // resume: an output file with the same header keeps its complete
    // records up to the first incomplete one
    int64_t done = 0;
    if (nml.resume) {
        done = complete_records(nml.datafile, hdr, rec, numeuler);
        if (done > 0) say(" resuming after %lld complete patterns\n", (long long)done);
    }
    RecordFile out(nml.datafile, rec * sizeof(float), done);
    if (!out.ok()) return fail(EBSD_EIO, std::string("cannot create output file '") + nml.datafile + "'");
    if (done == 0 && !out.write_header(hdr)) return fail(EBSD_EIO, "output header write failed");

    // contiguous shards of the remaining orientations, one per handle
    const auto t0 = std::chrono::steady_clock::now();                 // Time_start (:567)
    const int64_t left = numeuler - done;
    std::vector<int> shard_rc(ndev, EBSD_OK);
    std::vector<std::string> shard_err(ndev);
    {
        std::vector<std::thread> th;
        for (int k = 0; k < ndev; ++k) {
            const int64_t b = done + left * k / ndev, e = done + left * (k + 1) / ndev;
            th.emplace_back([&, k, b, e] {
                shard_rc[k] = run_shard(hg[k].h, devices[k], quats.data(), b, e, &epi, rec, &out,
                                        &shard_err[k]);
            });
        }
        for (auto& t : th) t.join();
    }
    for (int k = 0; k < ndev; ++k)
        if (shard_rc[k]) {
            char buf[64];
            snprintf(buf, sizeof buf, "device %d: ", devices[k]);
            return fail(shard_rc[k], buf + shard_err[k]);
        }
    if (!out.close()) return fail(EBSD_EIO, "output file write failed");
    const double secs =
        std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    say("  Total computation time [s] %.3f\n", secs);                 // Time_stop (:669)
    say("  Time per step/pixel [s] %10.6f\n", numeuler > 0 ? secs / (double)numeuler : 0.0);
    return EBSD_OK;
}

// The CTEMMC program on the GPU: CTEMMC.f90:48-277, the trajectory loop of
// single_run replaced by ebsd_mc_run, the MC file written as the reference
// writes it.  On several GPUs each device runs a contiguous range of the
// electrons into histograms of its own (every electron's random stream is
// keyed by its index in the whole run), and the host adds them up: integer
// sums, so the file is the one-device file byte for byte.
extern "C" int ebsd_run_mc_namelist(const char* nmlfile, int device, int quiet)
{
    const int32_t d = device;
    return ebsd_run_mc_namelist_devices(nmlfile, &d, 1, quiet);
}

extern "C" int ebsd_run_mc_namelist_devices(const char* nmlfile, const int32_t* devices,
                                            int32_t ndev, int quiet)
{
    if (!devices || ndev < 1 || ndev > 64)
        return fail(EBSD_EINVAL, "ebsd_run_mc_namelist_devices: 1 to 64 devices");
    auto say = [&](const char* fmt, auto... args) {
        if (!quiet) {
            printf(fmt, args...);
            fflush(stdout);
        }
    };
    say(" CTEMMC (GB300): Monte Carlo Electron Trajectory Simulation for EBSD+Lambert\n");
    ebsd_mc_namelist nml;
    std::string err;
    int rc = host::read_mc_namelist(nmlfile, &nml, &err);
    if (rc) return fail(rc, err);
    if (std::string(nml.xtalname) == "undefined")                       // :188-190
        return fail(EBSD_EINVAL, std::string("CTEMMC: structure file name is undefined in ") +
                                     nmlfile);
    if (std::string(nml.MCmode) != "CSDA")
        return fail(EBSD_EUNSUPPORTED, std::string("MCmode '") + nml.MCmode +
                                           "': only 'CSDA' exists in the reference");
    if (!(nml.density > 0.0) || !(nml.Ze > 0.0) || !(nml.at_wt > 0.0))
        return fail(EBSD_EUNSUPPORTED,
                    std::string("reading crystal files is not supported: give density, Ze and "
                                "at_wt in &MCdata (CTEMMC prints them as 'Density, avZ, avA' for ") +
                        nml.xtalname + ")");
    if (nml.num_el < 0 || nml.nthreads < 1) return fail(EBSD_EINVAL, "num_el, nthreads");
    say(" Density, avZ, avA = %10.5f%10.5f,%10.5f\n", nml.density, nml.Ze, nml.at_wt);
    ebsd_mc_params p;
    p.sig = nml.sig;
    p.omega = nml.omega;
    p.EkeV = nml.EkeV;
    p.Ehistmin = nml.Ehistmin;
    p.Ebinsize = nml.Ebinsize;
    p.depthmax = nml.depthmax;
    p.depthstep = nml.depthstep;
    p.Ze = nml.Ze;
    p.density = nml.density;
    p.at_wt = nml.at_wt;
    p.numsx = nml.numsx;
    int32_t nE = 0, nz = 0;
    rc = ebsd_mc_dims(&p, &nE, &nz);
    if (rc) return rc;
    const int nx = (nml.numsx - 1) / 2, n10 = nx / 10;
    const size_t ne = (size_t)nE * nml.numsx * nml.numsx;
    const size_t nzs = (size_t)nE * nz * (2 * n10 + 1) * (2 * n10 + 1);
    std::vector<int32_t> accum_e(ne);
    std::vector<int32_t> accum_z(nzs);
    std::vector<HandleGuard> hg(ndev);
    for (int k = 0; k < ndev; ++k) {
        rc = ebsd_create(&hg[k].h, devices[k]);
        if (rc) return rc;
    }
    const int64_t total = nml.num_el * (int64_t)nml.nthreads;
    say(" electrons: %lld x %d streams of the reference = %lld, one Philox stream each\n",
        (long long)nml.num_el, nml.nthreads, (long long)total);
    const auto t0 = std::chrono::steady_clock::now();
    int64_t counted = 0;
    {
        // device k: electrons [total*k/ndev, total*(k+1)/ndev) into its own
        // host histograms (device 0 straight into the result)
        std::vector<std::vector<int32_t>> pe(ndev - 1), pz(ndev - 1);
        std::vector<int64_t> cnt(ndev, 0);
        std::vector<int> rcs(ndev, EBSD_OK);
        std::vector<std::thread> th;
        for (int k = 0; k < ndev; ++k) {
            if (k > 0) {
                pe[k - 1].assign(ne, 0);
                pz[k - 1].assign(nzs, 0);
            }
            th.emplace_back([&, k] {
                const int64_t a = total * k / ndev, b = total * (k + 1) / ndev;
                int32_t* e = k ? pe[k - 1].data() : accum_e.data();
                int32_t* z = k ? pz[k - 1].data() : accum_z.data();
                rcs[k] = ebsd_mc_run(hg[k].h, &p, (uint64_t)(uint32_t)nml.primeseed, a, b - a, e,
                                     z, &cnt[k]);
            });
        }
        for (auto& t : th) t.join();
        for (int k = 0; k < ndev; ++k)
            if (rcs[k]) {
                host::global_set_error(rcs[k], ebsd_last_error(hg[k].h));
                return rcs[k];
            }
        for (int k = 0; k < ndev; ++k) counted += cnt[k];
        for (int k = 1; k < ndev; ++k) {
            for (size_t i = 0; i < ne; ++i) accum_e[i] += pe[k - 1][i];
            for (size_t i = 0; i < nzs; ++i) accum_z[i] += pz[k - 1][i];
        }
    }
    const double secs =
        std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    say("\n  All trajectories complete (%.3f s); saving data to file %s\n\n", secs,
        nml.dataname);
    say("  Total number of electrons generated = %lld\n", (long long)total);
    say("  Number of electrons on detector       = %lld\n", (long long)counted);

    host::FortranWriter out(nml.dataname);                              // :259-277
    if (!out.ok()) return fail(EBSD_EIO, std::string("cannot create ") + nml.dataname);
    auto chars = [](const char* sv, size_t n) {
        std::string r(sv);
        r.resize(n, ' ');
        return r;
    };
    const std::string prog = chars("CTEMMC.f90", 132), ver = chars("2.0/2013", 8),
                      xtal = chars(nml.xtalname, 132), mode = chars(nml.MCmode, 4);
    struct __attribute__((packed)) {
        int32_t a, b, c, d;
        int64_t n;
        int32_t t;
    } dims = {nE, nz, nml.numsx, nml.numsx, total, nml.nthreads};
    const double ener[5] = {nml.EkeV, nml.Ehistmin, nml.Ebinsize, nml.depthmax, nml.depthstep};
    const double tilt[2] = {nml.sig, nml.omega};
    bool ok = out.write(prog.data(), prog.size()) && out.write(ver.data(), ver.size()) &&
              out.write(xtal.data(), xtal.size()) && out.write(&dims, sizeof dims) &&
              out.write(ener, sizeof ener) && out.write(tilt, sizeof tilt) &&
              out.write(mode.data(), mode.size()) &&
              out.write(accum_e.data(), accum_e.size() * 4) &&
              out.write(accum_z.data(), accum_z.size() * 4);
    if (!ok || !out.close()) return fail(EBSD_EIO, "MC output file write failed");
    return EBSD_OK;
}
