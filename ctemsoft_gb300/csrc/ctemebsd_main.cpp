// ctemebsd: command-line drop-in for the CTEMEBSD program.
//
// Same command line as the reference (files.f90:623-688): an optional
// namelist file name (default CTEMEBSD.nml), -h for help and -t to write a
// namelist template into the current folder; any flag stops the program
// after it is handled.  One addition: -d N selects the CUDA device, and
// -d N,M,... splits the orientations over several devices.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/ebsd_gpu.h"

namespace {

const char* kTemplate =
    "&EBSDdata\n"
    "! CTEMEBSD namelist (GB300 drop-in); units as in the reference program\n"
    "! scintillator distance [microns]\n"
    " L = 15000.0\n"
    "! detector tilt below horizontal [degrees]\n"
    " thetac = 10.0\n"
    "! pixel size on the scintillator [microns]\n"
    " delta = 20.0\n"
    "! number of detector pixels along x and y\n"
    " numsx = 640\n"
    " numsy = 480\n"
    "! pattern centre [pixels]\n"
    " xpc = 0.0\n"
    " ypc = 0.0\n"
    "! angle file: first line 'eu' or 'qu', second line the count, then one row per entry\n"
    " anglefile = 'angles.txt'\n"
    "! Euler angle convention, 'tsl' or 'hkl'\n"
    " eulerconvention = 'tsl'\n"
    "! master pattern file (CTEMEBSDmaster output)\n"
    " FZfile = 'master.data'\n"
    "! Monte Carlo file (CTEMMC output)\n"
    " energyfile = 'MC.data'\n"
    "! output file\n"
    " datafile = 'EBSDout.data'\n"
    "! beam current [nA] and dwell time [microseconds]\n"
    " beamcurrent = 15.0\n"
    " dwelltime = 100.0\n"
    "! energy window [keV]\n"
    " energymin = 10.0\n"
    " energymax = 20.0\n"
    "! binning (1, 2, 4 or 8), scaling mode ('not', 'lin' or 'gam') and gamma exponent\n"
    " binning = 1\n"
    " scalingmode = 'not'\n"
    " gammavalue = 1.0\n"
    "! optional rotation applied to all orientations: axis (3) and angle [degrees]\n"
    " axisangle = 0.0, 0.0, 1.0, 0.0\n"
    "! Poisson noise (the reference always adds it) and its seed\n"
    " poisson = .TRUE.\n"
    " seed = 1\n"
    " /\n";

void usage(const char* prog)
{
    printf("\n Program should be called as follows: \n");
    printf("        %s -h -t [nmlfile]\n", prog);
    printf(" where nmlfile is an optional file name for the namelist file;\n\n");
    printf(" If absent, the default name 'CTEMEBSD.nml' will be used.\n");
    printf(" To create a template of the input file, type %s -t\n", prog);
    printf(" To produce this message, type %s -h\n", prog);
    printf(" -d N runs on CUDA device N (default 0); -d N,M,... splits the orientations\n");
    printf("    over several devices.\n\n");
}

}  // namespace

int main(int argc, char** argv)
{
    std::string nml = "CTEMEBSD.nml";
    bool halt = false;
    int nonflag = 0;
    std::vector<int32_t> devices;
    for (int i = 1; i < argc; ++i) {
        const char* a = argv[i];
        if (a[0] == '-') {
            if (!strcmp(a, "-h")) {
                usage(argv[0]);
                halt = true;
            } else if (!strcmp(a, "-t")) {
                printf("\nCreating program template files:\n");
                FILE* f = fopen("CTEMEBSD.template", "w");
                if (!f || fputs(kTemplate, f) < 0) {
                    fprintf(stderr, "cannot write CTEMEBSD.template\n");
                    return 1;
                }
                fclose(f);
                printf("  -> created template file CTEMEBSD.template\n");
                halt = true;
            } else if (!strcmp(a, "-d") && i + 1 < argc) {
                devices.clear();
                for (const char* p = argv[++i]; *p;) {
                    char* end = nullptr;
                    const long d = strtol(p, &end, 10);
                    if (end == p || d < 0 || d > 1024) {
                        fprintf(stderr, "bad device list %s\n", argv[i]);
                        return 1;
                    }
                    devices.push_back((int32_t)d);
                    p = *end == ',' ? end + 1 : end;
                    if (*end && *end != ',') {
                        fprintf(stderr, "bad device list %s\n", argv[i]);
                        return 1;
                    }
                }
            } else {
                fprintf(stderr, "unknown option %s\n", a);
                halt = true;
            }
        } else {
            nml = a;
            ++nonflag;
        }
    }
    if (halt) {
        printf("\nTo execute program, remove all flags except for nml input file name\n\n");
        return 0;
    }
    (void)nonflag;
    if (devices.empty()) devices.push_back(0);
    const int rc = ebsd_run_namelist_devices(nml.c_str(), devices.data(), (int32_t)devices.size(), 0);
    if (rc != EBSD_OK) {
        fprintf(stderr, "CTEMEBSD: %s (code %d)\n", ebsd_last_error(nullptr), rc);
        return 1;
    }
    return 0;
}
