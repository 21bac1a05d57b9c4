// Host-side set-up arithmetic and file formats.  Compiled with
// -ffp-contract=off so float expressions are evaluated as gfortran does
// (one rounding per operator, left to right).
#include "ebsd_host.h"

#include <cctype>
#include <unistd.h>
#include <cerrno>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <functional>
#include <sstream>

namespace ebsd {
namespace host {

namespace {
constexpr double kPi = 3.141592653589793238;  // constants.f90:70; Lambert.f90:239
constexpr float kDtor = 0.0174533f;           // CTEMEBSD.f90:150
}  // namespace

float lambert_scale(int n) { return (float)((double)(float)n / std::sqrt(kPi * 0.5)); }

float lambert_spi2_f() { return (float)(std::sqrt(kPi) * 0.5); }

void detector_angles(double sig, float thetac, float* ca, float* sa)
{
    const float s = (float)sig;                          // sig = MCsig (:345)
    const float t = (s - thetac) * kDtor;
    const float alp = (float)(0.5 * kPi - (double)t);    // :422
    *ca = cosf(alp);
    *sa = sinf(alp);
}

void energy_window(float energymin, float energymax, double Ehistmin, double Ebinsize,
                   int numEbins, int32_t* Emin, int32_t* Emax)
{
    int a = (int)std::lround(((double)energymin - Ehistmin) / Ebinsize) + 1;
    int b = (int)std::lround(((double)energymax - Ehistmin) / Ebinsize) + 1;
    a = a < 1 ? 1 : (a > numEbins ? numEbins : a);
    b = b < 1 ? 1 : (b > numEbins ? numEbins : b);
    *Emin = a;
    *Emax = b;
}

double prefactor(double beamcurrent, double dwelltime, int32_t num_el)
{
    const double nAmpere = 6.241e18;  // CTEMEBSD.f90:151
    return 0.25 * nAmpere * beamcurrent * dwelltime * 1.0e-15 / (double)num_el;
}

void quat_mult(const float x[4], const float y[4], float r[4])
{
    const float r0 = x[0] * y[0] - x[1] * y[1] - x[2] * y[2] - x[3] * y[3];
    const float r1 = x[0] * y[1] + x[1] * y[0] + x[2] * y[3] - x[3] * y[2];
    const float r2 = x[0] * y[2] - x[1] * y[3] + x[2] * y[0] + x[3] * y[1];
    const float r3 = x[0] * y[3] + x[1] * y[2] - x[2] * y[1] + x[3] * y[0];
    r[0] = r0;
    r[1] = r1;
    r[2] = r2;
    r[3] = r3;
}

void eu2qu(const float e[3], float q[4])
{
    const float h0 = 0.5f * e[0], h1 = 0.5f * e[1], h2 = 0.5f * e[2];
    const float cPhi = cosf(h1), sPhi = sinf(h1);
    const float cm = cosf(h0 - h2), sm = sinf(h0 - h2);
    const float cp = cosf(h0 + h2), sp = sinf(h0 + h2);
    const float s = cPhi * cp;
    if (s < 0.0f) {  // Northern hemisphere sign convention
        q[0] = -s;
        q[1] = sPhi * cm;
        q[2] = sPhi * sm;
        q[3] = cPhi * sp;
    } else {
        q[0] = s;
        q[1] = -(sPhi * cm);
        q[2] = -(sPhi * sm);
        q[3] = -(cPhi * sp);
    }
}

void ax2qu(const float a[4], float q[4])
{
    // orientation matrix of the axis-angle pair (rotations.f90:743-775) ...
    float m[3][3];
    const float c = cosf(a[3]), s = sinf(a[3]), omc = 1.0f - c;
    for (int i = 0; i < 3; ++i) m[i][i] = a[i] * a[i] * omc + c;
    float t = omc * a[0] * a[1];
    m[0][1] = t + s * a[2];
    m[1][0] = t - s * a[2];
    t = omc * a[1] * a[2];
    m[1][2] = t + s * a[0];
    m[2][1] = t - s * a[0];
    t = omc * a[2] * a[0];
    m[2][0] = t + s * a[1];
    m[0][2] = t - s * a[1];
    // ... converted to a unit quaternion (rotations.f90:1575-1604)
    q[0] = sqrtf(m[0][0] + m[1][1] + m[2][2] + 1.0f) / 2.0f;
    q[1] = sqrtf(fabsf(m[0][0] - m[1][1] - m[2][2] + 1.0f)) / 2.0f;
    q[2] = sqrtf(fabsf(-m[0][0] + m[1][1] - m[2][2] + 1.0f)) / 2.0f;
    q[3] = sqrtf(fabsf(-m[0][0] - m[1][1] + m[2][2] + 1.0f)) / 2.0f;
    if (m[2][1] - m[1][2] < 0.0f) q[1] = -q[1];
    if (m[0][2] - m[2][0] < 0.0f) q[2] = -q[2];
    if (m[1][0] - m[0][1] < 0.0f) q[3] = -q[3];
    float n = q[0] * q[0];
    n = n + q[1] * q[1];
    n = n + q[2] * q[2];
    n = n + q[3] * q[3];
    const float inv = 1.0f / sqrtf(n);
    for (int i = 0; i < 4; ++i) q[i] = inv * q[i];
}

// ----------------------------------------------------------------------
// Fortran unformatted sequential files

FortranReader::FortranReader(const char* path) : path_(path ? path : "")
{
    f_ = path ? fopen(path, "rb") : nullptr;
    if (!f_) err_ = "cannot open '" + path_ + "': " + strerror(errno);
}

FortranReader::~FortranReader()
{
    if (f_) fclose(f_);
}

bool FortranReader::next(std::vector<char>& buf)
{
    buf.clear();
    if (!f_) return false;
    for (;;) {
        int32_t head = 0, tail = 0;
        if (fread(&head, 4, 1, f_) != 1) {
            err_ = "unexpected end of file in '" + path_ + "'";
            return false;
        }
        const int64_t len = head < 0 ? -(int64_t)head : head;
        const size_t off = buf.size();
        buf.resize(off + (size_t)len);
        if (len > 0 && fread(buf.data() + off, 1, (size_t)len, f_) != (size_t)len) {
            err_ = "truncated record in '" + path_ + "'";
            return false;
        }
        if (fread(&tail, 4, 1, f_) != 1 || (tail < 0 ? -(int64_t)tail : tail) != len) {
            err_ = "bad record marker in '" + path_ + "'";
            return false;
        }
        if (head >= 0) return true;
    }
}

bool FortranReader::skip()
{
    std::vector<char> tmp;
    return next(tmp);
}

FortranWriter::FortranWriter(const char* path) { f_ = path ? fopen(path, "wb") : nullptr; }

FortranWriter::FortranWriter(const char* path, long long keep_bytes)
{
    f_ = path ? fopen(path, "r+b") : nullptr;
    if (!f_) return;
    // drop a partial trailing record, then append after the kept bytes
    if (fflush(f_) != 0 || ftruncate(fileno(f_), (off_t)keep_bytes) != 0 ||
        fseeko(f_, (off_t)keep_bytes, SEEK_SET) != 0) {
        fclose(f_);
        f_ = nullptr;
    }
}

FortranWriter::~FortranWriter() { close(); }

bool FortranWriter::write(const void* data, size_t bytes)
{
    if (!f_) return false;
    const size_t max_sub = 2147483639u;  // gfortran's largest sub-record
    const char* p = (const char*)data;
    size_t left = bytes;
    bool first = true;
    do {
        const size_t n = left > max_sub ? max_sub : left;
        const bool more = left > n;
        const int32_t head = more ? -(int32_t)n : (int32_t)n;
        const int32_t tail = first ? (int32_t)n : -(int32_t)n;
        if (fwrite(&head, 4, 1, f_) != 1) return false;
        if (n && fwrite(p, 1, n, f_) != n) return false;
        if (fwrite(&tail, 4, 1, f_) != 1) return false;
        p += n;
        left -= n;
        first = false;
    } while (left > 0);
    return true;
}

bool FortranWriter::close()
{
    if (!f_) return true;
    const bool ok = fclose(f_) == 0;
    f_ = nullptr;
    return ok;
}

// ----------------------------------------------------------------------
// Namelist &EBSDdata

namespace {

struct Tok {
    enum Kind { Word, Str, Eq, Comma, Slash, LPar, RPar, End } kind;
    std::string text;
};

std::vector<Tok> tokenize(const std::string& s)
{
    std::vector<Tok> out;
    size_t i = 0, n = s.size();
    while (i < n) {
        const char c = s[i];
        if (c == '!') {
            while (i < n && s[i] != '\n') ++i;
        } else if (isspace((unsigned char)c)) {
            ++i;
        } else if (c == '\'' || c == '"') {
            std::string v;
            ++i;
            while (i < n) {
                if (s[i] == c) {
                    if (i + 1 < n && s[i + 1] == c) {
                        v += c;
                        i += 2;
                        continue;
                    }
                    ++i;
                    break;
                }
                v += s[i++];
            }
            out.push_back({Tok::Str, v});
        } else if (c == '=') {
            out.push_back({Tok::Eq, "="});
            ++i;
        } else if (c == ',') {
            out.push_back({Tok::Comma, ","});
            ++i;
        } else if (c == '/') {
            out.push_back({Tok::Slash, "/"});
            ++i;
        } else if (c == '(') {
            out.push_back({Tok::LPar, "("});
            ++i;
        } else if (c == ')') {
            out.push_back({Tok::RPar, ")"});
            ++i;
        } else {
            std::string v;
            while (i < n && !isspace((unsigned char)s[i]) && s[i] != ',' && s[i] != '=' &&
                   s[i] != '/' && s[i] != '(' && s[i] != ')' && s[i] != '!')
                v += s[i++];
            out.push_back({Tok::Word, v});
        }
    }
    out.push_back({Tok::End, ""});
    return out;
}

std::string lower(std::string s)
{
    for (auto& c : s) c = (char)tolower((unsigned char)c);
    return s;
}

bool parse_real_f(const std::string& t, float* v)
{
    std::string u = t;
    for (auto& c : u)
        if (c == 'd' || c == 'D') c = 'e';
    char* end = nullptr;
    errno = 0;
    float x = strtof(u.c_str(), &end);
    if (end == u.c_str() || *end) return false;
    *v = x;
    return true;
}

bool parse_real_d(const std::string& t, double* v)
{
    std::string u = t;
    for (auto& c : u)
        if (c == 'd' || c == 'D') c = 'e';
    char* end = nullptr;
    double x = strtod(u.c_str(), &end);
    if (end == u.c_str() || *end) return false;
    *v = x;
    return true;
}

bool parse_int(const std::string& t, int64_t* v)
{
    char* end = nullptr;
    long long x = strtoll(t.c_str(), &end, 10);
    if (end == t.c_str() || *end) return false;
    *v = x;
    return true;
}

bool parse_logical(const std::string& t, int32_t* v)
{
    std::string u = lower(t);
    size_t k = u[0] == '.' ? 1 : 0;
    if (k >= u.size()) return false;
    if (u[k] == 't') {
        *v = 1;
        return true;
    }
    if (u[k] == 'f') {
        *v = 0;
        return true;
    }
    int64_t i;
    if (parse_int(t, &i)) {
        *v = i != 0;
        return true;
    }
    return false;
}

void set_str(char* dst, size_t cap, const std::string& v, size_t fortran_len)
{
    std::string w = v.substr(0, std::min(fortran_len, cap - 1));
    while (!w.empty() && w.back() == ' ') w.pop_back();  // trim() as the reference does
    snprintf(dst, cap, "%s", w.c_str());
}

// Expand repeat counts r*value into a flat value list.
bool expand_values(const std::vector<Tok>& vals, std::vector<std::string>* out)
{
    for (const auto& t : vals) {
        if (t.kind == Tok::Word) {
            const size_t star = t.text.find('*');
            if (star != std::string::npos) {
                int64_t r;
                if (!parse_int(t.text.substr(0, star), &r) || r < 1 || r > 1000000) return false;
                const std::string v = t.text.substr(star + 1);
                for (int64_t k = 0; k < r; ++k) out->push_back(v);
                continue;
            }
        }
        out->push_back(t.text);
    }
    return true;
}

// One namelist group (Fortran namelist input): calls assign(key, index,
// values) for every "name[(index)] = values" of &group ... / in order; index
// is -1 without a subscript.  assign returns EBSD_OK or an error code.
using Assign =
    std::function<int(const std::string&, int64_t, const std::vector<std::string>&)>;

int parse_group(const char* path, const char* group, const Assign& assign, std::string* err)
{
    std::ifstream in(path ? path : "");
    if (!in) {
        *err = std::string("cannot open namelist file '") + (path ? path : "") + "'";
        return EBSD_EIO;
    }
    std::stringstream ss;
    ss << in.rdbuf();
    const std::vector<Tok> toks = tokenize(ss.str());
    size_t i = 0;
    // find the group start &group (or $group)
    const std::string g = lower(group);
    for (; i < toks.size(); ++i) {
        if (toks[i].kind == Tok::Word) {
            const std::string w = lower(toks[i].text);
            if (w == "&" + g || w == "$" + g) break;
        }
    }
    if (i >= toks.size() || toks[i].kind == Tok::End) {
        *err = "namelist group &" + std::string(group) + " not found in '" + std::string(path) + "'";
        return EBSD_EFORMAT;
    }
    ++i;
    for (;;) {
        while (toks[i].kind == Tok::Comma) ++i;
        if (toks[i].kind == Tok::Slash || toks[i].kind == Tok::End) break;
        if (toks[i].kind == Tok::Word) {
            const std::string w = lower(toks[i].text);
            if (w == "&end" || w == "$end" || w == "&") break;
        }
        if (toks[i].kind != Tok::Word) {
            *err = "namelist: expected a variable name, found '" + toks[i].text + "'";
            return EBSD_EFORMAT;
        }
        const std::string key = lower(toks[i].text);
        ++i;
        int64_t index = -1;
        if (toks[i].kind == Tok::LPar) {
            if (toks[i + 1].kind != Tok::Word || !parse_int(toks[i + 1].text, &index) ||
                toks[i + 2].kind != Tok::RPar) {
                *err = "namelist: bad subscript for '" + key + "'";
                return EBSD_EFORMAT;
            }
            i += 3;
        }
        if (toks[i].kind != Tok::Eq) {
            *err = "namelist: expected '=' after '" + key + "'";
            return EBSD_EFORMAT;
        }
        ++i;
        // values run until the next "name =", "name(" or the terminator
        std::vector<Tok> vals;
        for (;;) {
            const Tok& t = toks[i];
            if (t.kind == Tok::Slash || t.kind == Tok::End) break;
            if (t.kind == Tok::Word &&
                (toks[i + 1].kind == Tok::Eq || toks[i + 1].kind == Tok::LPar))
                break;
            if (t.kind == Tok::Word) {
                const std::string w = lower(t.text);
                if (w == "&end" || w == "$end") break;
            }
            if (t.kind != Tok::Comma) vals.push_back(t);
            ++i;
        }
        std::vector<std::string> v;
        if (!expand_values(vals, &v) || v.empty()) {
            *err = "namelist: no value for '" + key + "'";
            return EBSD_EFORMAT;
        }
        const int rc = assign(key, index, v);
        if (rc) return rc;
    }
    return EBSD_OK;
}

}  // namespace

int read_namelist(const char* path, ebsd_namelist* nml, std::string* err)
{
    // defaults of CTEMEBSD.f90:179-198
    memset(nml, 0, sizeof *nml);
    nml->L = 20000.0f;
    nml->thetac = 0.0f;
    nml->delta = 25.0f;
    nml->numsx = 640;
    nml->numsy = 480;
    nml->xpc = 0.0f;
    nml->ypc = 0.0f;
    nml->energymin = 15.0f;
    nml->energymax = 30.0f;
    snprintf(nml->anglefile, sizeof nml->anglefile, "euler.txt");
    snprintf(nml->eulerconvention, sizeof nml->eulerconvention, "tsl");
    snprintf(nml->FZfile, sizeof nml->FZfile, "FZ.data");
    snprintf(nml->energyfile, sizeof nml->energyfile, "energy.data");
    snprintf(nml->datafile, sizeof nml->datafile, "EBSDout.data");
    nml->beamcurrent = 14.513;
    nml->dwelltime = 100.0;
    snprintf(nml->scalingmode, sizeof nml->scalingmode, "not");
    nml->gammavalue = 1.0f;
    nml->binning = 1;
    nml->poisson = 1;
    nml->seed = 1;
    nml->resume = 0;
    nml->ncubochoric = 0;
    nml->pgnum = 32;
    return parse_group(path, "EBSDdata", [&](const std::string& key, int64_t index,
                                             const std::vector<std::string>& v) -> int {
        bool ok = true;
        auto f32 = [&](float* dst) { ok = v.size() == 1 && parse_real_f(v[0], dst); };
        auto f64 = [&](double* dst) { ok = v.size() == 1 && parse_real_d(v[0], dst); };
        auto i32 = [&](int32_t* dst) {
            int64_t x;
            ok = v.size() == 1 && parse_int(v[0], &x) && x >= INT32_MIN && x <= INT32_MAX;
            if (ok) *dst = (int32_t)x;
        };
        if (key == "l") f32(&nml->L);
        else if (key == "thetac") f32(&nml->thetac);
        else if (key == "delta") f32(&nml->delta);
        else if (key == "numsx") i32(&nml->numsx);
        else if (key == "numsy") i32(&nml->numsy);
        else if (key == "xpc") f32(&nml->xpc);
        else if (key == "ypc") f32(&nml->ypc);
        else if (key == "energymin") f32(&nml->energymin);
        else if (key == "energymax") f32(&nml->energymax);
        else if (key == "beamcurrent") f64(&nml->beamcurrent);
        else if (key == "dwelltime") f64(&nml->dwelltime);
        else if (key == "binning") i32(&nml->binning);
        else if (key == "gammavalue") f32(&nml->gammavalue);
        else if (key == "anglefile") set_str(nml->anglefile, sizeof nml->anglefile, v[0], 132);
        else if (key == "eulerconvention")
            set_str(nml->eulerconvention, sizeof nml->eulerconvention, v[0], 3);
        else if (key == "fzfile") set_str(nml->FZfile, sizeof nml->FZfile, v[0], 132);
        else if (key == "energyfile") set_str(nml->energyfile, sizeof nml->energyfile, v[0], 132);
        else if (key == "datafile") set_str(nml->datafile, sizeof nml->datafile, v[0], 132);
        else if (key == "scalingmode") set_str(nml->scalingmode, sizeof nml->scalingmode, v[0], 3);
        else if (key == "axisangle") {
            if (index >= 1) {
                ok = index <= 4 && v.size() == 1 && parse_real_f(v[0], &nml->axisangle[index - 1]);
            } else {
                ok = v.size() <= 4;
                for (size_t k = 0; ok && k < v.size(); ++k)
                    ok = parse_real_f(v[k], &nml->axisangle[k]);
            }
        } else if (key == "poisson") {
            ok = v.size() == 1 && parse_logical(v[0], &nml->poisson);
        } else if (key == "resume") {
            ok = v.size() == 1 && parse_logical(v[0], &nml->resume);
        } else if (key == "ncubochoric") {
            i32(&nml->ncubochoric);
        } else if (key == "pgnum") {
            i32(&nml->pgnum);
        } else if (key == "seed") {
            int64_t x;
            ok = v.size() == 1 && parse_int(v[0], &x);
            if (ok) nml->seed = x;
        } else {
            *err = "namelist: unknown variable '" + key + "' in group EBSDdata";
            return EBSD_EFORMAT;
        }
        if (!ok) {
            *err = "namelist: bad value for '" + key + "'";
            return EBSD_EFORMAT;
        }
        return EBSD_OK;
    }, err);
}

int read_mc_namelist(const char* path, ebsd_mc_namelist* nml, std::string* err)
{
    // defaults of CTEMMC.f90:171-183
    memset(nml, 0, sizeof *nml);
    snprintf(nml->MCmode, sizeof nml->MCmode, "CSDA");
    snprintf(nml->xtalname, sizeof nml->xtalname, "undefined");
    nml->sig = 70.0;
    nml->omega = 0.0;
    nml->numsx = 1501;
    nml->primeseed = 932117;
    nml->num_el = 10000000;
    nml->nthreads = 4;
    nml->EkeV = 30.0;
    nml->Ehistmin = 30.0 - 10.0;  // EkeV - 10 with the default EkeV, before the read
    nml->Ebinsize = 0.25;
    nml->depthmax = 50.0;
    nml->depthstep = 1.0;
    snprintf(nml->dataname, sizeof nml->dataname, "undefined.data");
    return parse_group(path, "MCdata", [&](const std::string& key, int64_t,
                                           const std::vector<std::string>& v) -> int {
        bool ok = true;
        auto f64 = [&](double* dst) { ok = v.size() == 1 && parse_real_d(v[0], dst); };
        auto i32 = [&](int32_t* dst) {
            int64_t x;
            ok = v.size() == 1 && parse_int(v[0], &x) && x >= INT32_MIN && x <= INT32_MAX;
            if (ok) *dst = (int32_t)x;
        };
        if (key == "xtalname") set_str(nml->xtalname, sizeof nml->xtalname, v[0], 132);
        else if (key == "sig") f64(&nml->sig);
        else if (key == "omega") f64(&nml->omega);
        else if (key == "numsx") i32(&nml->numsx);
        else if (key == "num_el") {
            int64_t x;
            ok = v.size() == 1 && parse_int(v[0], &x);
            if (ok) nml->num_el = x;
        } else if (key == "primeseed") i32(&nml->primeseed);
        else if (key == "ekev") f64(&nml->EkeV);
        else if (key == "dataname") set_str(nml->dataname, sizeof nml->dataname, v[0], 60);
        else if (key == "nthreads") i32(&nml->nthreads);
        else if (key == "ehistmin") f64(&nml->Ehistmin);
        else if (key == "ebinsize") f64(&nml->Ebinsize);
        else if (key == "depthmax") f64(&nml->depthmax);
        else if (key == "depthstep") f64(&nml->depthstep);
        else if (key == "mcmode") set_str(nml->MCmode, sizeof nml->MCmode, v[0], 4);
        else if (key == "density") f64(&nml->density);
        else if (key == "ze") f64(&nml->Ze);
        else if (key == "at_wt") f64(&nml->at_wt);
        else {
            *err = "namelist: unknown variable '" + key + "' in group MCdata";
            return EBSD_EFORMAT;
        }
        if (!ok) {
            *err = "namelist: bad value for '" + key + "'";
            return EBSD_EFORMAT;
        }
        return EBSD_OK;
    }, err);
}

// ----------------------------------------------------------------------
// Angle file, CTEMEBSD.f90:228-288 (list-directed reads)

namespace {

// One list-directed READ: starts at the next line and consumes `count`
// values, continuing onto following lines; a '/' ends the read early.
bool list_read(std::istream& in, size_t count, std::vector<std::string>* vals)
{
    vals->clear();
    std::string line;
    while (vals->size() < count) {
        if (!std::getline(in, line)) return false;
        size_t i = 0;
        while (i < line.size() && vals->size() < count) {
            const char c = line[i];
            if (isspace((unsigned char)c) || c == ',') {
                ++i;
                continue;
            }
            if (c == '/') return true;
            if (c == '\'' || c == '"') {
                std::string v;
                ++i;
                while (i < line.size() && line[i] != c) v += line[i++];
                ++i;
                vals->push_back(v);
                continue;
            }
            std::string v;
            while (i < line.size() && !isspace((unsigned char)line[i]) && line[i] != ',' &&
                   line[i] != '/')
                v += line[i++];
            vals->push_back(v);
        }
    }
    return true;
}

}  // namespace

int read_angle_file(const char* path, const char* conv, const float axisangle[4],
                    std::vector<float>* quats, std::string* err)
{
    std::ifstream in(path ? path : "");
    if (!in) {
        *err = std::string("cannot open angle file '") + (path ? path : "") + "'";
        return EBSD_EIO;
    }
    std::vector<std::string> v;
    if (!list_read(in, 1, &v) || v.empty()) {
        *err = "angle file: missing angle type";
        return EBSD_EFORMAT;
    }
    const std::string type = v[0].substr(0, 2);
    const bool euler = type == "eu";
    if (!list_read(in, 1, &v) || v.empty()) {
        *err = "angle file: missing number of angles";
        return EBSD_EFORMAT;
    }
    int64_t n;
    if (!parse_int(v[0], &n) || n < 0) {
        *err = "angle file: bad number of angles '" + v[0] + "'";
        return EBSD_EFORMAT;
    }
    quats->assign((size_t)n * 4, 0.0f);
    const bool hkl = conv && std::string(conv).substr(0, 3) == "hkl";
    for (int64_t i = 0; i < n; ++i) {
        const size_t m = euler ? 3 : 4;
        if (!list_read(in, m, &v) || v.size() != m) {
            *err = "angle file: too few rows or values at entry " + std::to_string(i + 1);
            return EBSD_EFORMAT;
        }
        float r[4];
        for (size_t k = 0; k < m; ++k)
            if (!parse_real_f(v[k], &r[k])) {
                *err = "angle file: bad number '" + v[k] + "'";
                return EBSD_EFORMAT;
            }
        float* q = quats->data() + 4 * i;
        if (euler) {
            if (hkl) r[0] = r[0] + 90.0f;                             // :256
            const float e[3] = {r[0] * kDtor, r[1] * kDtor, r[2] * kDtor};  // :267
            eu2qu(e, q);
        } else {
            memcpy(q, r, sizeof(float) * 4);
        }
    }
    apply_axisangle(axisangle, quats->data(), n);
    return EBSD_OK;
}

void apply_axisangle(const float axisangle[4], float* quats, int64_t n)
{
    if (!axisangle || axisangle[3] == 0.0f) return;                  // :282-288
    const float a[4] = {axisangle[0], axisangle[1], axisangle[2], axisangle[3] * kDtor};
    float qax[4];
    ax2qu(a, qax);
    for (int64_t i = 0; i < n; ++i) {
        float r[4];
        quat_mult(qax, quats + 4 * i, r);
        memcpy(quats + 4 * i, r, sizeof r);
    }
}

// ----------------------------------------------------------------------
// MC file (CTEMMC.f90:262-277, read as CTEMEBSD.f90:319-355)

int read_mc_file(const char* path, ebsd_mc_header* hdr, std::vector<int32_t>* accum_e,
                 int32_t* dst, std::string* err)
{
    FortranReader r(path);
    if (!r.ok()) {
        *err = r.error();
        return EBSD_EIO;
    }
    std::vector<char> b;
    for (int k = 0; k < 3; ++k)  // progname, scversion, xtalname
        if (!r.next(b)) {
            *err = r.error();
            return EBSD_EFORMAT;
        }
    if (!r.next(b) || b.size() < 24) {
        *err = "MC file: short header record";
        return EBSD_EFORMAT;
    }
    memset(hdr, 0, sizeof *hdr);
    memcpy(&hdr->numEbins, b.data(), 4);
    memcpy(&hdr->numzbins, b.data() + 4, 4);
    memcpy(&hdr->numsx, b.data() + 8, 4);
    memcpy(&hdr->numsy, b.data() + 12, 4);
    if (b.size() >= 28) {
        memcpy(&hdr->num_el_total, b.data() + 16, 8);
        memcpy(&hdr->nthreads, b.data() + 24, 4);
    } else {
        int32_t ne;
        memcpy(&ne, b.data() + 16, 4);
        hdr->num_el_total = ne;
        memcpy(&hdr->nthreads, b.data() + 20, 4);
    }
    if (!r.next(b) || b.size() < 40) {
        *err = "MC file: short energy record";
        return EBSD_EFORMAT;
    }
    memcpy(&hdr->EkeV, b.data(), 8);
    memcpy(&hdr->Ehistmin, b.data() + 8, 8);
    memcpy(&hdr->Ebinsize, b.data() + 16, 8);
    memcpy(&hdr->depthmax, b.data() + 24, 8);
    memcpy(&hdr->depthstep, b.data() + 32, 8);
    if (!r.next(b) || b.size() < 16) {
        *err = "MC file: short tilt record";
        return EBSD_EFORMAT;
    }
    memcpy(&hdr->sig, b.data(), 8);
    memcpy(&hdr->omega, b.data() + 8, 8);
    if (!r.next(b) || b.size() < 4) {
        *err = "MC file: missing MCmode record";
        return EBSD_EFORMAT;
    }
    memcpy(hdr->MCmode, b.data(), 4);
    hdr->MCmode[4] = 0;
    if (hdr->numEbins < 1 || hdr->numsx < 1 || hdr->numsy < 1) {
        *err = "MC file: non-positive dimensions";
        return EBSD_EFORMAT;
    }
    if (!accum_e && !dst) return EBSD_OK;
    const int nsx = (hdr->numsx - 1) / 2, nsy = (hdr->numsy - 1) / 2;  // :333-334
    const size_t count = (size_t)hdr->numEbins * (2 * nsx + 1) * (2 * nsy + 1);
    if (!r.next(b) || b.size() < count * 4) {
        *err = "MC file: accum_e record shorter than numEbins*(2nsx+1)*(2nsy+1)";
        return EBSD_EFORMAT;
    }
    if (accum_e) {
        accum_e->resize(count);
        memcpy(accum_e->data(), b.data(), count * 4);
    }
    if (dst) memcpy(dst, b.data(), count * 4);
    return EBSD_OK;
}

// ----------------------------------------------------------------------
// Master file (CTEMEBSDmaster.f90:540-568, read as CTEMEBSD.f90:378-406)

int read_master_file(const char* path, ebsd_master_header* hdr, float* EkeVs, int32_t* atomtype,
                     float* srtmp, std::vector<float>* srvec, std::string* err)
{
    FortranReader r(path);
    if (!r.ok()) {
        *err = r.error();
        return EBSD_EIO;
    }
    std::vector<char> b;
    for (int k = 0; k < 4; ++k)  // progname, scversion, xtalname, energyfile
        if (!r.next(b)) {
            *err = r.error();
            return EBSD_EFORMAT;
        }
    if (!r.next(b) || b.size() < 16) {
        *err = "master file: short dimension record";
        return EBSD_EFORMAT;
    }
    memset(hdr, 0, sizeof *hdr);
    memcpy(&hdr->npx, b.data(), 4);
    memcpy(&hdr->npy, b.data() + 4, 4);
    memcpy(&hdr->nE, b.data() + 8, 4);
    memcpy(&hdr->numset, b.data() + 12, 4);
    if (hdr->npx < 1 || hdr->npy < 1 || hdr->nE < 1 || hdr->numset < 1) {
        *err = "master file: non-positive dimensions";
        return EBSD_EFORMAT;
    }
    if (!r.next(b) || b.size() < (size_t)hdr->nE * 4) {
        *err = "master file: short energy record";
        return EBSD_EFORMAT;
    }
    if (EkeVs) memcpy(EkeVs, b.data(), (size_t)hdr->nE * 4);
    if (!r.next(b) || b.size() < (size_t)hdr->numset * 4) {
        *err = "master file: short atom type record";
        return EBSD_EFORMAT;
    }
    if (atomtype) memcpy(atomtype, b.data(), (size_t)hdr->numset * 4);
    if (!r.next(b) || b.size() < 6) {
        *err = "master file: missing projection type record";
        return EBSD_EFORMAT;
    }
    memcpy(hdr->sqorhe, b.data(), 6);
    hdr->sqorhe[6] = 0;
    if (!srtmp && !srvec) return EBSD_OK;
    const size_t count =
        (size_t)(2 * hdr->npx + 1) * (2 * hdr->npy + 1) * hdr->nE * hdr->numset;
    if (!r.next(b) || b.size() < count * 4) {
        *err = "master file: pattern record shorter than (2npx+1)*(2npy+1)*nE*numset";
        return EBSD_EFORMAT;
    }
    if (srtmp) memcpy(srtmp, b.data(), count * 4);
    if (srvec) {
        srvec->resize(count);
        memcpy(srvec->data(), b.data(), count * 4);
    }
    return EBSD_OK;
}

}  // namespace host
}  // namespace ebsd

// ----------------------------------------------------------------------
// C ABI wrappers for the file readers

using namespace ebsd;

extern "C" int ebsd_read_mc_file(const char* path, ebsd_mc_header* hdr, int32_t* accum_e)
{
    if (!hdr) return host::global_set_error(EBSD_EINVAL, "ebsd_read_mc_file: null header");
    std::string err;
    int rc = host::read_mc_file(path, hdr, nullptr, accum_e, &err);
    if (rc) host::global_set_error(rc, err.c_str());
    return rc;
}

extern "C" int ebsd_read_master_file(const char* path, ebsd_master_header* hdr, float* EkeVs,
                                     int32_t* atomtype, float* srtmp)
{
    if (!hdr) return host::global_set_error(EBSD_EINVAL, "ebsd_read_master_file: null header");
    std::string err;
    int rc = host::read_master_file(path, hdr, EkeVs, atomtype, srtmp, nullptr, &err);
    if (rc) host::global_set_error(rc, err.c_str());
    return rc;
}

extern "C" int ebsd_read_namelist(const char* path, ebsd_namelist* nml)
{
    if (!nml) return host::global_set_error(EBSD_EINVAL, "ebsd_read_namelist: null output");
    std::string err;
    int rc = host::read_namelist(path, nml, &err);
    if (rc) host::global_set_error(rc, err.c_str());
    return rc;
}

extern "C" int ebsd_read_mc_namelist(const char* path, ebsd_mc_namelist* nml)
{
    if (!nml) return host::global_set_error(EBSD_EINVAL, "ebsd_read_mc_namelist: null output");
    std::string err;
    int rc = host::read_mc_namelist(path, nml, &err);
    if (rc) host::global_set_error(rc, err.c_str());
    return rc;
}

extern "C" int ebsd_read_angle_file(const char* path, const char* eulerconvention,
                                    const float axisangle[4], int64_t* n, float* quats)
{
    if (!n) return host::global_set_error(EBSD_EINVAL, "ebsd_read_angle_file: null count");
    std::vector<float> q;
    std::string err;
    int rc = host::read_angle_file(path, eulerconvention, axisangle, &q, &err);
    if (rc) {
        host::global_set_error(rc, err.c_str());
        return rc;
    }
    const int64_t have = (int64_t)(q.size() / 4);
    if (quats) {
        if (*n < have)
            return host::global_set_error(EBSD_EINVAL,
                                          "ebsd_read_angle_file: output holds fewer quaternions "
                                          "than the file");
        memcpy(quats, q.data(), q.size() * sizeof(float));
    }
    *n = have;
    return EBSD_OK;
}
