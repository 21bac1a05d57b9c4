// The CTEMEBSD program on the GPU: CTEMEBSD.f90:87-672 end to end, with the
// pattern loop replaced by libebsdgpu calls and the output written by a
// writer thread while the next chunk of patterns is computed.
#include <cuda_runtime.h>

#include <algorithm>
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

extern "C" int ebsd_run_namelist(const char* nmlfile, int device, int quiet)
{
    auto say = [&](const char* fmt, auto... args) {
        if (!quiet) {
            printf(fmt, args...);
            fflush(stdout);
        }
    };
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

    HandleGuard hg;
    rc = ebsd_create(&hg.h, device);
    if (rc) return rc;
    ebsd_handle* h = hg.h;
    auto herr = [&](int code) {
        host::global_set_error(code, ebsd_last_error(h));
        return code;
    };
    if (dictionary) {
        int64_t cnt = 0;
        rc = ebsd_sample_rfz(h, nml.ncubochoric, nml.pgnum, nullptr, nullptr, 0, &cnt);
        if (rc) return herr(rc);
        quats.resize((size_t)cnt * 4);
        rc = ebsd_sample_rfz(h, nml.ncubochoric, nml.pgnum, nullptr, quats.data(), cnt, &cnt);
        if (rc) return herr(rc);
        host::apply_axisangle(nml.axisangle, quats.data(), cnt);
        numeuler = cnt;
        say(" Cubochoric sampling, %d steps, point group %d: %lld orientations in the "
            "fundamental zone\n", nml.ncubochoric, nml.pgnum, (long long)numeuler);
    }
    rc = ebsd_set_master(h, srtmp.data(), mh.npx, mh.npy, mh.nE, mh.numset);
    if (rc) return herr(rc);
    srtmp.clear();
    srtmp.shrink_to_fit();

    ebsd_geometry g;
    g.L = nml.L;
    g.thetac = nml.thetac;
    g.delta = nml.delta;
    g.numsx = nml.numsx;
    g.numsy = nml.numsy;
    g.xpc = nml.xpc;
    g.ypc = nml.ypc;
    g.sig = mc.sig;
    int32_t num_el = 0;
    rc = ebsd_set_detector(h, &g, accum_e.data(), nsx, nsy, mc.numEbins, Emin, Emax, &num_el);
    if (rc) return herr(rc);
    accum_e.clear();
    accum_e.shrink_to_fit();

    const double pref = host::prefactor(nml.beamcurrent, nml.dwelltime, num_el);
    {
        std::vector<float> W((size_t)mc.numEbins * g.numsx * g.numsy);
        rc = ebsd_get_detector(h, W.data(), nullptr, nullptr, nullptr);
        if (rc) return herr(rc);
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
    if (rc) return herr(rc);

    // output header (:555-561): binned dimensions whenever binning != 1
    int32_t hdr[3] = {nml.numsx, nml.numsy, (int32_t)numeuler};
    if (nml.binning != 1) {
        hdr[0] = nml.numsx / nml.binning;
        hdr[1] = nml.numsy / nml.binning;
    }
    const size_t rec = (size_t)rx * ry;
    // resume: an output file with the same header keeps its complete
    // records (20-byte header record, then 4*rec + 8 bytes per pattern)
    int64_t done = 0;
    if (nml.resume) {
        FILE* f = fopen(nml.datafile, "rb");
        if (f) {
            int32_t head[5] = {0, 0, 0, 0, 0};
            const bool hok = fread(head, 4, 5, f) == 5 && head[0] == 12 && head[4] == 12 &&
                             head[1] == hdr[0] && head[2] == hdr[1] && head[3] == hdr[2];
            fseeko(f, 0, SEEK_END);
            const long long size = (long long)ftello(f);
            fclose(f);
            if (hok) {
                const long long per = 4LL * (long long)rec + 8;
                done = std::min<int64_t>(numeuler, (size - 20) / per);
                while (done > 0) {  // the last counted record must be complete
                    FILE* g2 = fopen(nml.datafile, "rb");
                    int32_t m1 = 0, m2 = 0;
                    const long long off = 20 + (done - 1) * per;
                    bool ok2 = g2 && fseeko(g2, off, SEEK_SET) == 0 && fread(&m1, 4, 1, g2) == 1 &&
                               fseeko(g2, off + 4 + 4LL * (long long)rec, SEEK_SET) == 0 &&
                               fread(&m2, 4, 1, g2) == 1;
                    if (g2) fclose(g2);
                    if (ok2 && m1 == (int32_t)(4 * rec) && m2 == m1) break;
                    --done;
                }
                say(" resuming after %lld complete patterns\n", (long long)done);
            }
        }
    }
    std::unique_ptr<host::FortranWriter> outp;
    if (done > 0)
        outp.reset(new host::FortranWriter(nml.datafile, 20 + done * (4LL * (long long)rec + 8)));
    else
        outp.reset(new host::FortranWriter(nml.datafile));
    host::FortranWriter& out = *outp;
    if (!out.ok()) return fail(EBSD_EIO, std::string("cannot create output file '") + nml.datafile + "'");
    if (done == 0 && !out.write(hdr, sizeof hdr)) return fail(EBSD_EIO, "output header write failed");

    const auto t0 = std::chrono::steady_clock::now();                 // Time_start (:567)
    const int64_t chunk = std::max<int64_t>(
        1, std::min<int64_t>(numeuler, (int64_t)((size_t(256) << 20) / (rec * sizeof(float)))));
    PinnedGuard pg;
    for (int b = 0; b < 2; ++b) {
        cudaError_t e = cudaMallocHost(&pg.p[b], std::max<size_t>(1, chunk * rec) * sizeof(float));
        if (e != cudaSuccess) return fail(EBSD_ENOMEM, "pinned output buffer");
    }
    std::thread writer;
    bool write_ok = true;
    for (int64_t o0 = done, c = 0; o0 < numeuler; o0 += chunk, ++c) {
        const int64_t m = std::min(chunk, numeuler - o0);
        float* buf = pg.p[c & 1];
        rc = ebsd_forward(h, quats.data() + 4 * o0, m, &epi, buf);
        if (rc) {
            if (writer.joinable()) writer.join();
            return herr(rc);
        }
        if (writer.joinable()) writer.join();
        writer = std::thread([&out, &write_ok, buf, m, rec] {
            for (int64_t k = 0; k < m && write_ok; ++k)                // one record per pattern
                write_ok = out.write(buf + (size_t)k * rec, rec * sizeof(float));
        });
    }
    if (writer.joinable()) writer.join();
    if (!write_ok || !out.close()) return fail(EBSD_EIO, "output file write failed");
    const double secs =
        std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    say("  Total computation time [s] %.3f\n", secs);                 // Time_stop (:669)
    say("  Time per step/pixel [s] %10.6f\n", numeuler > 0 ? secs / (double)numeuler : 0.0);
    return EBSD_OK;
}

// The CTEMMC program on the GPU: CTEMMC.f90:48-277, the trajectory loop of
// single_run replaced by ebsd_mc_run, the MC file written as the reference
// writes it.
extern "C" int ebsd_run_mc_namelist(const char* nmlfile, int device, int quiet)
{
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
    std::vector<int32_t> accum_e((size_t)nE * nml.numsx * nml.numsx);
    std::vector<int32_t> accum_z((size_t)nE * nz * (2 * n10 + 1) * (2 * n10 + 1));
    HandleGuard hg;
    rc = ebsd_create(&hg.h, device);
    if (rc) return rc;
    const int64_t total = nml.num_el * (int64_t)nml.nthreads;
    say(" electrons: %lld x %d streams of the reference = %lld, one Philox stream each\n",
        (long long)nml.num_el, nml.nthreads, (long long)total);
    const auto t0 = std::chrono::steady_clock::now();
    int64_t counted = 0;
    rc = ebsd_mc_run(hg.h, &p, (uint64_t)(uint32_t)nml.primeseed, 0, total, accum_e.data(),
                     accum_z.data(), &counted);
    if (rc) {
        host::global_set_error(rc, ebsd_last_error(hg.h));
        return rc;
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
