// ctemmc: command-line drop-in for the CTEMMC program.
//
// Same command line as the reference (files.f90:623-688): an optional
// namelist file name (default CTEMMC.nml), -h for help and -t to write a
// namelist template into the current folder; any flag stops the program
// after it is handled.  One addition: -d N selects the CUDA device, and
// -d N,M,... splits the electrons over several devices.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/ebsd_gpu.h"

namespace {

const char* kTemplate =
    "&MCdata\n"
    "! CTEMMC namelist (GB300 drop-in); units as in the reference program\n"
    "! crystal structure name (written to the output header)\n"
    " xtalname = 'Ni.xtal'\n"
    "! the crystal's density [g/cm^3], average atomic number and average atomic\n"
    "! weight [g/mol] (the reference computes these from the crystal file)\n"
    " density = 8.908\n"
    " Ze = 28.0\n"
    " at_wt = 58.6934\n"
    "! sample tilt angles sigma (about TD) and omega (about RD) [degrees]\n"
    " sig = 70.0\n"
    " omega = 0.0\n"
    "! number of points along the side of the modified Lambert grid (odd)\n"
    " numsx = 1501\n"
    "! electrons per thread, and threads: num_el*nthreads electrons in total\n"
    " num_el = 10000000\n"
    " nthreads = 4\n"
    "! random number seed\n"
    " primeseed = 932117\n"
    "! beam energy, lowest energy bin and bin size [keV]\n"
    " EkeV = 20.0\n"
    " Ehistmin = 10.0\n"
    " Ebinsize = 1.0\n"
    "! exit-depth histogram: deepest bin and bin size [nm]\n"
    " depthmax = 100.0\n"
    " depthstep = 1.0\n"
    "! Monte Carlo mode\n"
    " MCmode = 'CSDA'\n"
    "! output file\n"
    " dataname = 'MC.data'\n"
    " /\n";

void usage(const char* prog)
{
    printf("\n Program should be called as follows: \n");
    printf("        %s -h -t [nmlfile]\n", prog);
    printf(" where nmlfile is an optional file name for the namelist file;\n\n");
    printf(" If absent, the default name 'CTEMMC.nml' will be used.\n");
    printf(" To create a template of the input file, type %s -t\n", prog);
    printf(" To produce this message, type %s -h\n", prog);
    printf(" -d N runs on CUDA device N (default 0); -d N,M,... splits the electrons\n");
    printf("    over several devices.\n\n");
}

}  // namespace

int main(int argc, char** argv)
{
    std::string nml = "CTEMMC.nml";
    bool halt = false;
    std::vector<int32_t> devices;
    for (int i = 1; i < argc; ++i) {
        const char* a = argv[i];
        if (a[0] == '-') {
            if (!strcmp(a, "-h")) {
                usage(argv[0]);
                halt = true;
            } else if (!strcmp(a, "-t")) {
                printf("\nCreating program template files:\n");
                FILE* f = fopen("CTEMMC.template", "w");
                if (!f || fputs(kTemplate, f) < 0) {
                    fprintf(stderr, "cannot write CTEMMC.template\n");
                    return 1;
                }
                fclose(f);
                printf("  -> created template file CTEMMC.template\n");
                halt = true;
            } else if (!strcmp(a, "-d") && i + 1 < argc) {
                devices.clear();
                for (const char* q = argv[++i]; *q;) {
                    char* end = nullptr;
                    const long d = strtol(q, &end, 10);
                    if (end == q || d < 0 || d > 1024 || (*end && *end != ',')) {
                        fprintf(stderr, "bad device list %s\n", argv[i]);
                        return 1;
                    }
                    devices.push_back((int32_t)d);
                    q = *end == ',' ? end + 1 : end;
                }
            } else {
                fprintf(stderr, "unknown option %s\n", a);
                halt = true;
            }
        } else {
            nml = a;
        }
    }
    if (halt) {
        printf("\nTo execute program, remove all flags except for nml input file name\n\n");
        return 0;
    }
    if (devices.empty()) devices.push_back(0);
    const int rc =
        ebsd_run_mc_namelist_devices(nml.c_str(), devices.data(), (int32_t)devices.size(), 0);
    if (rc != EBSD_OK) {
        fprintf(stderr, "CTEMMC: %s (code %d)\n", ebsd_last_error(nullptr), rc);
        return 1;
    }
    return 0;
}
