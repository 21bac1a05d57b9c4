// Host-side pieces of libebsdgpu.so: the reference's scalar set-up
// arithmetic, Fortran unformatted sequential files, the &EBSDdata namelist
// and angle files.
#pragma once

#include <stdint.h>
#include <stdio.h>

#include <string>
#include <vector>

#include "../../include/ebsd_gpu.h"

namespace ebsd {
namespace host {

// sngl(float(n)/LPs%sPio2): CTEMEBSD.f90:481,571 (binary64 divide, rounded).
float lambert_scale(int n);
// sngl(LPs%sPi2): Lambert.f90:243-245,428.
float lambert_spi2_f();
// ca, sa of CTEMEBSD.f90:422-424 (alp mixes binary64 cPi with sgl angles).
void detector_angles(double sig, float thetac, float* ca, float* sa);
// CTEMEBSD.f90:361-367.
void energy_window(float energymin, float energymax, double Ehistmin, double Ebinsize,
                   int numEbins, int32_t* Emin, int32_t* Emax);
// CTEMEBSD.f90:545.
double prefactor(double beamcurrent, double dwelltime, int32_t num_el);
// rotations.f90:1322-1351 eu2qu (radians), single precision.
void eu2qu(const float e[3], float q[4]);
// rotations.f90:2116-2124 ax2qu (axis, angle in radians), single precision.
void ax2qu(const float a[4], float q[4]);
// quaternions.f90:255-264.
void quat_mult(const float x[4], const float y[4], float r[4]);

// Fortran unformatted sequential file (gfortran layout: 4-byte record
// markers; records over 2 GiB split into signed sub-records).
class FortranReader {
public:
    explicit FortranReader(const char* path);
    ~FortranReader();
    bool ok() const { return f_ != nullptr; }
    // Reads the next record into buf; returns false at EOF or on a
    // malformed marker (error() says which).
    bool next(std::vector<char>& buf);
    // Skips one record.
    bool skip();
    const std::string& error() const { return err_; }

private:
    FILE* f_ = nullptr;
    std::string err_;
    std::string path_;
};

class FortranWriter {
public:
    explicit FortranWriter(const char* path);
    // Re-open an existing file, truncate it to keep_bytes and append there.
    FortranWriter(const char* path, long long keep_bytes);
    ~FortranWriter();
    bool ok() const { return f_ != nullptr; }
    bool write(const void* data, size_t bytes);
    bool close();

private:
    FILE* f_ = nullptr;
};

int read_namelist(const char* path, ebsd_namelist* nml, std::string* err);
int read_mc_namelist(const char* path, ebsd_mc_namelist* nml, std::string* err);
int read_angle_file(const char* path, const char* conv, const float axisangle[4],
                    std::vector<float>* quats, std::string* err);
// q <- qax (x) q for n quaternions when axisangle(4) != 0 (CTEMEBSD.f90:282-288).
void apply_axisangle(const float axisangle[4], float* quats, int64_t n);
int read_mc_file(const char* path, ebsd_mc_header* hdr, std::vector<int32_t>* accum_e,
                 int32_t* dst, std::string* err);
int read_master_file(const char* path, ebsd_master_header* hdr, float* EkeVs, int32_t* atomtype,
                     float* srtmp, std::vector<float>* srvec, std::string* err);

// Handle internals used by the program driver.
float handle_max_sr(const ebsd_handle* h);
int handle_set_error(ebsd_handle* h, int code, const char* msg);
int global_set_error(int code, const char* msg);

}  // namespace host
}  // namespace ebsd
