// fd23_psv2d: the reference's P-SV program (PN nbpsv2d and its topabsorb /
// explosion builds, PD psv2d_db without the box) on the fd23 engine; built
// with FD23_CLI_SH=1 it is fd23_sh2d, the reference's SH program (SH/main.cpp).
//
//   fd23_psv2d par=run.par [key=value ...]
//   fd23_sh2d  par=run.par [key=value ...]
//
// SH differences (SH/param/param.cpp:13-85): the source time function key is
// "sourcetime" (srctime is accepted too), "stype" selects the source (3
// moment, 13 'p' dipole; 2, the line force on V, is an addition), receivers
// come from V_sta_file or nrec ixrec0 izrec0_v idxrec idzrec, and the output
// is <output>_V with <output>_V.isis (no position shift).  ngpu is accepted.
//
// Parameters follow the reference's parameter reader (PN/param/param.cpp:88-200,
// getpar conventions): key=value words on the command line, "par=file" reads
// key=value words from a file at that point (# starts a comment), and the
// last value given for a key wins.  Required: nx nz nt h dt srctime (with
// alpha for Gaussian, trap1 trap2 trap3 for Trapezoid) strike dip rake
// azimuth xs zs npml pml_dt pml_v pml_r pml_fc output model, and either
// U_sta_file / W_sta_file or nrec ixrec0 izrec0_u izrec0_w idxrec idzrec.
// Optional: srctype (1 moment, p 'p' dipole; default 1), itrecord (1),
// restart + nt0, savestate.  Accepted and ignored (no effect on this path):
// ntsnap itprint gpuid ngpu ord bw sourcetime stype; src_shift_x and
// src_shift_z (default 0.25, -0.25) only enter the FP64 trace headers.  usepunch=1 (with before, after, timefile) updates
// every 32 x 16 tile only inside its step window (PN/slide/cu_slide.cu,
// PN/param/param.cpp usepunch block): the timefile holds nx*nz float travel
// times (PN, SH), or doubles with prec=f64 (PD, whose windows use the double
// dt).  usetable=1 (PN/param/param.cpp:180-181; the SH program's default,
// SH/main.cpp:154) reads the material through a table of its distinct
// tuples when they fit (fd23_set_material_table), else prints the
// reference's "Too many materials" and goes on without.  usebox=1 (P-SV,
// prec f32 or f64; PD/main.cpp:153-200, PD/box/box.cpp) runs the hybrid
// box of width bw around (xs, zs) instead of the point source: the box
// material is the homogeneous srcpvel / srcsvel / srcden
// (PD/material/material.cpp:39-97, box cells of the model that differ are
// replaced), and the incident field comes from sourcefile, the
// displacement planes the box-source generator wrote (fd23_ntde_line or
// the reference's ntde_line), read frame by frame as the reference reads
// them (a frame past the end of the file leaves the older buffer in place,
// PD/box/box.cpp:120-139); boxsource=device (an addition) generates the
// planes on the GPU from the parfile's source instead of reading the file.
// zs closer than bw/2+4 to the top or bottom is refused
// (PD/param/param.cpp:182-185).  Additions: prec (f32, f64,
// bf16, f16; default f32; f64 reads h and dt as doubles, as the PD
// programs do, the others round them to float as PN does),
// explosion (1: Mxx = Mzz = 1, the *_exp builds), topabsorb (1: CPML on top,
// the *_topabsorb builds), device (CUDA ordinal, default 0), dryrun (1: print
// the resolved set-up and stop before touching the GPU).
//
// Outputs as the reference writes them (PN/main.cpp:216-230, 253-326,
// PN/record/isis.cpp): <output>_U and <output>_W, raw [recorded step][trace]
// in the compute type (float, double for f64); <output>_U.isis and
// <output>_W.isis, one 84-byte trace header and the float trace per
// receiver (U positions shifted +0.5 cell in x, W -0.5 cell in z); with
// savestate=1 the state file state%06d (step nt0+nt-1); with restart=1 the
// run starts from state%06d (step nt0-1).  Header words the reference leaves
// unset are written as zero.  With prec=f64 the trace files are the FP64
// program's (PD/record/isis.cpp:8-58): <output>_U.db.isis and
// <output>_W.db.isis, a 136-byte double header and the double trace per
// receiver, the source position shifted by src_shift_x / src_shift_z cells,
// user[1] = bw (0 without the box), user[2] = 123456789.
//
// Built with FD23_CLI_NTDE=1 it is fd23_ntde_line, the reference's
// box-source generator (PD/source/source_line.cpp:307-410): from the same
// parfile (nt h dt srcden srcsvel srcpvel sourcefile bw sourcetime with
// alpha or trap1-3, strike dip rake azimuth; device optional) it writes
// sourcefile, nt frames of the (bw+8) x (bw+8) U and W displacement planes
// as doubles, computed on the GPU (fd23_line_source_planes).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/fd23.h"

#ifndef FD23_CLI_SH
#define FD23_CLI_SH 0
#endif
#ifndef FD23_CLI_NTDE
#define FD23_CLI_NTDE 0
#endif

namespace {

constexpr bool kSH = FD23_CLI_SH != 0;
constexpr bool kNTDE = FD23_CLI_NTDE != 0;
const char *kProg = kNTDE ? "fd23_ntde_line" : (kSH ? "fd23_sh2d" : "fd23_psv2d");

struct Params {
    std::map<std::string, std::string> kv;
    std::vector<std::string> missing;

    bool has(const std::string &k) const { return kv.count(k) != 0; }
    std::string str(const std::string &k, const std::string &d = "")
    {
        auto it = kv.find(k);
        if (it != kv.end()) return it->second;
        return d;
    }
    std::string need(const std::string &k)
    {
        if (!has(k)) {
            missing.push_back(k);
            return "0";
        }
        return kv[k];
    }
    double num(const std::string &k, double d) { return has(k) ? std::atof(kv[k].c_str()) : d; }
    double need_num(const std::string &k) { return std::atof(need(k).c_str()); }
};

bool add_word(Params &p, const std::string &w)
{
    const size_t e = w.find('=');
    if (e == std::string::npos || e == 0) return false;
    p.kv[w.substr(0, e)] = w.substr(e + 1);
    return true;
}

bool load_parfile(Params &p, const std::string &path)
{
    std::ifstream f(path);
    if (!f) return false;
    for (std::string line; std::getline(f, line);) {
        const size_t c = line.find('#');
        if (c != std::string::npos) line.resize(c);
        std::istringstream is(line);
        for (std::string w; is >> w;)
            if (!add_word(p, w)) return false;
    }
    return true;
}

// 84-byte trace header of the .isis trace files (PN/record/isis.h)
struct IsisTrace {
    float xs, ys, zs;
    float xr, yr, zr;
    float t0;
    int nt;
    float samplerate;
    int srcflagnum, recflagnum, status;
    float gain, dtstatic, ampstatic;
    unsigned short recorder, chan, scomp, rcomp;
    int user[4];
};
static_assert(sizeof(IsisTrace) == 84, "isis trace header is 84 bytes");

// 136-byte trace header of the FP64 program's trace files
// (PD/record/isis.h:7-26): the same words in double, with the natural
// alignment padding after nt and after status
struct IsisTraceDb {
    double xs, ys, zs;
    double xr, yr, zr;
    double t0;
    int nt;
    double samplerate;
    int srcflagnum, recflagnum, status;
    double gain, dtstatic, ampstatic;
    unsigned short recorder, chan, scomp, rcomp;
    int user[4];
};
static_assert(sizeof(IsisTraceDb) == 136, "FP64 isis trace header is 136 bytes");

int fail(const char *what, int rc)
{
    std::fprintf(stderr, "%s: %s: %s\n", kProg, what, fd23_strerror(rc));
    return 1;
}

bool write_file(const std::string &name, const void *p, size_t bytes)
{
    std::ofstream f(name, std::ios::binary);
    return f && f.write((const char *)p, (std::streamsize)bytes);
}

bool report_missing(Params &p)
{
    if (p.missing.empty()) return false;
    std::fprintf(stderr, "%s: missing parameter(s):", kProg);
    for (auto &m : p.missing) std::fprintf(stderr, " %s", m.c_str());
    std::fprintf(stderr, "\n");
    return true;
}

// the source time function of the PD programs' "sourcetime" keys
// (PD/param/param.cpp:92-100): s(t)*dt samples, or an empty vector
std::vector<double> pd_wavelet(Params &p, double dt)
{
    const std::string st = p.need("sourcetime");
    std::vector<double> src(1 << 20);
    int n = -1;
    if (!st.empty() && (st[0] == 'G' || st[0] == 'g'))
        n = fd23_wavelet_gaussian(dt, (int)p.need_num("alpha"), src.data(), (int)src.size());
    else if (!st.empty() && (st[0] == 'T' || st[0] == 't'))
        n = fd23_wavelet_trapezoid(dt, p.need_num("trap1"), p.need_num("trap2"), p.need_num("trap3"), src.data(),
                                   (int)src.size());
    src.resize(n > 0 ? n : 0);
    return src;
}

// the line source of the box-source generator for a bw x bw box around its
// source (PD/source/source_line.cpp:307-347)
fd23_line_desc line_desc(int bw, double h, double dt, double vp, double vs, double den, double strike, double dip,
                         double rake, double azimuth)
{
    fd23_line_desc d{};
    d.px = d.pz = bw + 8;
    d.ox = d.oz = fd23_line_plane_origin(bw);
    d.h = h;
    d.dt = dt;
    d.vp = vp;
    d.vs = vs;
    d.den = den;
    fd23_line_source_coefs(strike, dip, rake, azimuth, d.a);
    d.sx = 0.25;  // the generator's fixed source point (source_line.cpp:309-310)
    d.sz = -0.25;
    return d;
}

// fd23_ntde_line: the planes of frames 0 .. nt-1 into sourcefile
int ntde_main(Params &p)
{
    const int nt = (int)p.need_num("nt"), bw = (int)p.need_num("bw");
    const double h = p.need_num("h"), dt = p.need_num("dt");
    const double den = p.need_num("srcden"), vs = p.need_num("srcsvel"), vp = p.need_num("srcpvel");
    const std::string out = p.need("sourcefile");
    const double strike = p.need_num("strike"), dip = p.need_num("dip"), rake = p.need_num("rake"),
                 azimuth = p.need_num("azimuth");
    const std::vector<double> src = pd_wavelet(p, dt);
    const int device = (int)p.num("device", 0);
    if (report_missing(p)) return 1;
    if (src.empty() || nt < 1 || bw < 1) {
        std::fprintf(stderr, "%s: sourcetime must be Gaussian or Trapezoid; nt and bw positive\n", kProg);
        return 1;
    }
    const fd23_line_desc d = line_desc(bw, h, dt, vp, vs, den, strike, dip, rake, azimuth);
    const size_t frame = 2 * (size_t)d.px * d.pz;
    std::ofstream f(out, std::ios::binary);
    if (!f) {
        std::fprintf(stderr, "%s: cannot write %s\n", kProg, out.c_str());
        return 1;
    }
    const int chunk = (int)std::max<size_t>(1, ((size_t)64 << 20) / (frame * sizeof(double)));
    std::vector<double> buf;
    for (int f0 = 0; f0 < nt; f0 += chunk) {
        const int nf = std::min(chunk, nt - f0);
        buf.resize((size_t)nf * frame);
        const int rc = fd23_line_source_planes(device, &d, src.data(), (int)src.size(), f0, nf, buf.data());
        if (rc) return fail("planes", rc);
        if (!f.write((const char *)buf.data(), (std::streamsize)(buf.size() * sizeof(double)))) {
            std::fprintf(stderr, "%s: cannot write %s\n", kProg, out.c_str());
            return 1;
        }
    }
    std::printf("finish!\n");
    return 0;
}

// The box's incident field of steps 0 .. nt-1 from the planes file, read as
// BOX::init_box / setboxsource read it (PD/box/box.cpp:106-139): frame 0 at
// set-up, one frame per step into alternating buffers; a read past the end
// of the file leaves the buffer as it was.
int incident_from_file(const std::string &name, int bw, int nt, double dt, const std::vector<double> &bmat,
                       bool f64, std::vector<unsigned char> &inc)
{
    int nsub = 0, nadd = 0;
    const int nring = fd23_box_ring_size(bw, bw, &nsub, &nadd);
    if (nring < 0) return nring;
    const size_t plane = (size_t)(bw + 8) * (bw + 8);
    std::ifstream f(name, std::ios::binary);
    if (!f) return FD23_ERR_ARG;
    std::vector<double> u1(plane), w1(plane), u2(plane), w2(plane), one(5 * (size_t)nring);
    auto rd = [&](std::vector<double> &v) {
        if (f) f.read((char *)v.data(), (std::streamsize)(plane * sizeof(double)));
    };
    rd(u1);
    rd(w1);
    if (!f) return FD23_ERR_ARG;  // not even frame 0
    const size_t cs = f64 ? 8 : 4;
    inc.assign((size_t)nt * 5 * nring * cs, 0);
    bool read_u1 = false;
    for (int it = 0; it < nt; ++it) {
        std::vector<double> &un = read_u1 ? u1 : u2, &wn = read_u1 ? w1 : w2;
        const std::vector<double> &uo = read_u1 ? u2 : u1, &wo = read_u1 ? w2 : w1;
        rd(un);
        rd(wn);
        read_u1 = !read_u1;
        const int rc = fd23_box_incident_from_displacement(bw, bw, dt, bmat.data(), uo.data(), wo.data(),
                                                           un.data(), wn.data(), one.data());
        if (rc < 0) return rc;
        unsigned char *o = inc.data() + (size_t)it * 5 * nring * cs;
        for (size_t k = 0; k < one.size(); ++k) {
            if (f64) reinterpret_cast<double *>(o)[k] = one[k];
            else reinterpret_cast<float *>(o)[k] = (float)one[k];
        }
    }
    return FD23_OK;
}

}  // namespace

int main(int argc, char **argv)
{
    Params p;
    for (int i = 1; i < argc; ++i) {
        const std::string a(argv[i]);
        if (a.rfind("par=", 0) == 0) {
            if (!load_parfile(p, a.substr(4))) {
                std::fprintf(stderr, "%s: ", kProg); std::fprintf(stderr, "cannot read parameter file %s\n", a.substr(4).c_str());
                return 1;
            }
        } else if (!add_word(p, a)) {
            std::fprintf(stderr, "%s: ", kProg); std::fprintf(stderr, "expected key=value, got '%s'\n", a.c_str());
            return 1;
        }
    }
    if (argc < 2) {
        std::fprintf(stderr, "usage: %s par=file [key=value ...]\n", kProg);
        return 1;
    }
    if (kNTDE) return ntde_main(p);
    const std::string precs = p.str("prec", "f32");
    const int restart = (int)p.num("restart", 0), savestate = (int)p.num("savestate", 0);
    const int nt0 = restart ? (int)p.need_num("nt0") : 0;
    const int nx = (int)p.need_num("nx"), nz = (int)p.need_num("nz"), nt = (int)p.need_num("nt");
    // PN reads h and dt as float, PD (prec=f64) as double
    const bool pd = precs == "f64";
    const double h = pd ? p.need_num("h") : (double)(float)p.need_num("h");
    const double dt = pd ? p.need_num("dt") : (double)(float)p.need_num("dt");
    const float hf = (float)h, dtf = (float)dt;
    const std::string srctype = p.str("srctype", "1");
    const int stype = (int)p.num("stype", 3);
    // SH and PD name the key sourcetime, PN srctime; either is accepted
    const std::string srctime = p.has("srctime") && !(kSH && p.has("sourcetime"))
                                    ? p.str("srctime")
                                    : (p.has("sourcetime") || kSH ? p.need("sourcetime") : p.need("srctime"));
    double alpha = 0, trap[3] = {0, 0, 0};
    if (!srctime.empty() && (srctime[0] == 'T' || srctime[0] == 't'))
        for (int k = 0; k < 3; ++k) trap[k] = p.need_num("trap" + std::to_string(k + 1));
    if (!srctime.empty() && (srctime[0] == 'G' || srctime[0] == 'g')) alpha = p.need_num("alpha");
    const double strike = p.need_num("strike"), dip = p.need_num("dip"), rake = p.need_num("rake"),
                 azimuth = p.need_num("azimuth");
    const int xs = (int)p.need_num("xs"), zs = (int)p.need_num("zs");
    const double src_shift_x = p.num("src_shift_x", 0.25), src_shift_z = p.num("src_shift_z", -0.25);
    const int npml = (int)p.need_num("npml");
    const double pml_dt = p.need_num("pml_dt"), pml_v = p.need_num("pml_v"), pml_r = p.need_num("pml_r"),
                 pml_fc = p.need_num("pml_fc");
    const int itrecord = (int)p.num("itrecord", 1);
    const std::string output = p.need("output");
    const std::string ufile = p.str(kSH ? "V_sta_file" : "U_sta_file"), wfile = kSH ? "" : p.str("W_sta_file");
    int nrec = 0, ixrec0 = 0, izu = 0, izw = 0, idx = 0, idz = 0;
    if (ufile.empty() && wfile.empty()) {
        nrec = (int)p.need_num("nrec");
        ixrec0 = (int)p.need_num("ixrec0");
        izu = (int)p.need_num(kSH ? "izrec0_v" : "izrec0_u");
        izw = kSH ? izu : (int)p.need_num("izrec0_w");
        idx = (int)p.need_num("idxrec");
        idz = (int)p.need_num("idzrec");
    }
    const std::string model = p.need("model");
    const int explosion = (int)p.num("explosion", 0), topabsorb = (int)p.num("topabsorb", 0);
    const int device = (int)p.num("device", 0);
    if (!p.missing.empty()) {
        std::fprintf(stderr, "%s: ", kProg); std::fprintf(stderr, "missing parameter(s):");
        for (auto &m : p.missing) std::fprintf(stderr, " %s", m.c_str());
        std::fprintf(stderr, "\n");
        return 1;
    }
    const int usebox = (int)p.num("usebox", 0);
    int bw = 0;
    double srcden = 0, srcsvel = 0, srcpvel = 0;
    std::string sourcefile;
    const bool box_device = p.str("boxsource", "file") == "device";
    if (usebox == 1) {
        srcden = p.need_num("srcden");
        srcsvel = p.need_num("srcsvel");
        srcpvel = p.need_num("srcpvel");
        bw = (int)p.need_num("bw");
        if (!box_device) sourcefile = p.need("sourcefile");
        if (report_missing(p)) return 1;
        if (kSH || (precs != "f32" && precs != "f64")) {
            std::fprintf(stderr, "%s: usebox=1 needs the P-SV program with prec f32 or f64\n", kProg);
            return 1;
        }
        if (zs < bw / 2 + 4 || nz - zs < bw / 2 + 4) {
            std::fprintf(stderr, "%s: zs %d is too near to the boundary\n", kProg, zs);
            return 1;
        }
        if (restart || savestate || p.num("usepunch", 0) != 0 || p.num("usetable", 0) != 0) {
            std::fprintf(stderr, "%s: usebox=1 runs without restart, savestate, usepunch and usetable\n", kProg);
            return 1;
        }
    }
    const int usepunch = (int)p.num("usepunch", 0);
    double before = 0, after = 0;
    std::string timefile;
    if (usepunch == 1) {
        before = p.need_num("before");
        after = p.need_num("after");
        timefile = p.need("timefile");
        if (!p.missing.empty()) {
            std::fprintf(stderr, "%s: ", kProg); std::fprintf(stderr, "usepunch=1 needs before, after and timefile\n");
            return 1;
        }
    }
    int prec = FD23_F32;
    if (precs == "f64") prec = FD23_F64;
    else if (precs == "bf16") prec = FD23_BF16;
    else if (precs == "f16") prec = FD23_F16;
    else if (precs != "f32") {
        std::fprintf(stderr, "%s: ", kProg); std::fprintf(stderr, "prec must be f32, f64, bf16 or f16\n");
        return 1;
    }
    if (!kSH && srctype != "1" && srctype != "p" && srctype != "P") {
        std::fprintf(stderr, "%s: ", kProg); std::fprintf(stderr, "Wrong srctype! Specify 1 or p.\n");
        return 1;
    }
    if (kSH && stype != 3 && stype != 13 && stype != 2) {
        std::fprintf(stderr, "%s: ", kProg); std::fprintf(stderr, "stype must be 3, 13 or 2\n");
        return 1;
    }
    if (srctime.empty() || !std::strchr("GgTt", srctime[0])) {
        std::fprintf(stderr, "%s: ", kProg); std::fprintf(stderr, "srctime must be Gaussian or Trapezoid\n");
        return 1;
    }
    // source time function: s(t)*dt samples
    std::vector<double> src(1 << 20);
    const int lsrc = (srctime[0] == 'G' || srctime[0] == 'g')
                         ? fd23_wavelet_gaussian(dt, (int)alpha, src.data(), (int)src.size())
                         : fd23_wavelet_trapezoid(dt, trap[0], trap[1], trap[2], src.data(), (int)src.size());
    if (lsrc <= 0) return fail("source time function", lsrc < 0 ? lsrc : FD23_ERR_ARG);
    // receivers
    std::vector<int> rxu, rzu, rxw, rzw;
    auto stations = [](const std::string &f, std::vector<int> &rx, std::vector<int> &rz) -> int {
        const int n = fd23_read_stations(f.c_str(), nullptr, nullptr, 0);
        if (n < 0) return n;
        rx.resize(n);
        rz.resize(n);
        return fd23_read_stations(f.c_str(), rx.data(), rz.data(), n);
    };
    if (!ufile.empty() || !wfile.empty()) {
        int rc = stations(ufile.empty() ? wfile : ufile, rxu, rzu);
        if (rc < 0) return fail(("station file " + ufile).c_str(), rc);
        if ((rc = stations(wfile.empty() ? ufile : wfile, rxw, rzw)) < 0)
            return fail(("station file " + wfile).c_str(), rc);
    } else {
        rxu.resize(2 * nrec);
        rzu.resize(2 * nrec);
        rxw.resize(2 * nrec);
        rzw.resize(2 * nrec);
        fd23_receivers_line(nrec, ixrec0, izu, idx, idz, rxu.data(), rzu.data());
        fd23_receivers_line(nrec, ixrec0, izw, idx, idz, rxw.data(), rzw.data());
    }
    // tile step windows
    int nbx = 0, nbz = 0;
    std::vector<int> pfirst, plast;
    if (usepunch == 1) {
        fd23_punch_tiles(nx, nz, &nbx, &nbz);
        pfirst.resize((size_t)nbx * nbz);
        plast.resize((size_t)nbx * nbz);
        const int es = precs == "f64" ? 8 : 4;
        const double pdt = es == 8 ? p.need_num("dt") : (double)dt;
        const int rc = fd23_read_punch(timefile.c_str(), es, nx, nz, before, after, pdt, pfirst.data(), plast.data());
        if (rc) return fail(("timefile " + timefile).c_str(), rc);
    }
    if (p.num("dryrun", 0) != 0) {
        std::printf("{\"nx\": %d, \"nz\": %d, \"nt\": %d, \"nt0\": %d, \"h\": %.9g, \"dt\": %.9g, \"npml\": %d, "
                    "\"topabsorb\": %d, \"prec\": \"%s\", \"source\": \"%s\", \"xs\": %d, \"zs\": %d, "
                    "\"lsrc\": %d, \"itrecord\": %d, \"traces_u\": %zu, \"traces_w\": %zu, \"model\": \"%s\", "
                    "\"output\": \"%s\", \"savestate\": %d, \"punch_tiles\": %d, \"punch_first_min\": %d, "
                    "\"box\": [%d, %d, %d, %d], \"boxsource\": \"%s\"}\n",
                    nx, nz, nt, nt0, h, dt, npml, topabsorb, precs.c_str(),
                    kSH ? (stype == 2 ? "force" : (stype == 13 ? "moment_p" : "moment"))
                        : (explosion ? "explosion" : (srctype == "1" ? "moment" : "moment_p")),
                    xs, zs, lsrc, itrecord,
                    rxu.size(), rxw.size(), model.c_str(), output.c_str(), savestate, nbx * nbz,
                    pfirst.empty() ? 0 : *std::min_element(pfirst.begin(), pfirst.end()),
                    usebox == 1 ? xs + (bw + 1) / 2 + 1 - bw : 0, usebox == 1 ? zs + (bw + 1) / 2 + 1 - bw : 0,
                    usebox == 1 ? bw : 0, usebox == 1 ? bw : 0,
                    usebox != 1 ? "none" : (box_device ? "device" : sourcefile.c_str()));
        return 0;
    }
    // model
    const size_t n = (size_t)nx * nz;
    std::vector<double> vp(n), vs(n), den(n);
    int rc = fd23_read_model(model.c_str(), nx, nz, h, vp.data(), vs.data(), den.data());
    if (rc) return fail(("model " + model).c_str(), rc);
    fd23_desc d{};
    d.wave = kSH ? FD23_SH : FD23_PSV;
    d.prec = prec;
    d.nx = nx;
    d.nz = nz;
    d.npml = npml;
    d.topabsorb = topabsorb;
    d.h = h;
    d.dt = dt;
    d.pml_dt = pml_dt;
    d.pml_v = pml_v;
    d.pml_r = pml_r;
    d.pml_fc = pml_fc;
    d.device = device;
    d.kernel = FD23_KERNEL_AUTO;
    fd23_solver *s = nullptr;
    if ((rc = fd23_create(&d, &s))) return fail("create", rc);
    double stab = 0;
    std::vector<double> bmat;
    const int bx0 = xs + (bw + 1) / 2 + 1 - bw, bz0 = zs + (bw + 1) / 2 + 1 - bw;  // PD/box/box.cpp:26-45
    if (usebox == 1) {
        // the grid material with the box made homogeneous, and the box's own
        // (MATERIAL::get_model then BOX::init_box, PD/main.cpp:229-236)
        std::vector<double> mat(5 * n);
        rc = fd23_build_material(FD23_PSV, nx, nz, h, dt, vp.data(), vs.data(), den.data(), mat.data(), &stab);
        std::printf("stab = %g\n", stab);
        if (rc) return fail("model", rc);
        bmat.resize(5 * (size_t)bw * bw);
        rc = fd23_box_material(nx, nz, mat.data(), bx0, bz0, bw, bw, srcpvel, srcsvel, srcden, dt, h, bmat.data());
        if (rc < 0) return fail("box material", rc);
        if ((rc = fd23_set_material(s, mat.data()))) return fail("material", rc);
        if ((rc = fd23_set_box(s, bx0, bz0, bw, bw, bmat.data()))) return fail("box", rc);
    } else {
        rc = fd23_set_model(s, kSH ? nullptr : vp.data(), vs.data(), den.data(), &stab);
        std::printf("stab = %g\n", stab);
        if (rc) return fail("model", rc);
    }
    // material table (PN/param/param.cpp usetable; the SH program always
    // tries one, SH/main.cpp:154): index + table form when the distinct
    // material tuples fit, the material arrays otherwise
    if (p.num("usetable", kSH ? 1 : 0) != 0) {
        rc = fd23_set_material_table(s, 1);
        if (rc == FD23_ERR_UNSUPPORTED) std::printf("Too many materials, abort make table\n");
        else if (rc < 0) return fail("material table", rc);
        else std::printf("material table: %d entries\n", rc);
    }
    double m[3];
    int kind;
    if (kSH) {
        fd23_moment_sh(strike, dip, rake, azimuth, m);
        kind = stype == 2 ? FD23_SRC_FORCE : (stype == 13 ? FD23_SRC_MOMENT_P : FD23_SRC_MOMENT);
    } else {
        fd23_moment_psv(strike, dip, rake, azimuth, m);
        kind = explosion ? FD23_SRC_EXPLOSION : (srctype == "1" ? FD23_SRC_MOMENT : FD23_SRC_MOMENT_P);
    }
    if (usebox == 1) {
        // the box is the source (PD/main.cpp:153-200 has no point source)
        if (box_device) {
            const fd23_line_desc ld = line_desc(bw, h, dt, srcpvel, srcsvel, srcden, strike, dip, rake, azimuth);
            if ((rc = fd23_set_box_line_source(s, &ld, src.data(), lsrc, bmat.data(), 0, nt)))
                return fail("box source", rc);
        } else {
            std::vector<unsigned char> inc;
            if ((rc = incident_from_file(sourcefile, bw, nt, dt, bmat, prec == FD23_F64, inc)))
                return fail(("sourcefile " + sourcefile).c_str(), rc);
            if ((rc = fd23_set_box_incident(s, inc.data(), 0, nt))) return fail("box incident", rc);
        }
    } else if ((rc = fd23_set_source(s, kind, xs, zs, m, src.data(), lsrc, nt0 + nt))) {
        return fail("source", rc);
    }
    if ((rc = fd23_set_receivers(s, 0, rxu.data(), rzu.data(), (int)rxu.size()))) return fail("receivers", rc);
    if (!kSH && (rc = fd23_set_receivers(s, FD23_W, rxw.data(), rzw.data(), (int)rxw.size())))
        return fail("W receivers", rc);
    if (usepunch == 1 && (rc = fd23_set_punch(s, pfirst.data(), plast.data(), nbx, nbz)))
        return fail("usepunch", rc);
    const size_t sbytes = fd23_state_bytes(s);
    char statefile[64];
    if (restart) {
        std::snprintf(statefile, sizeof statefile, "state%06d", nt0 - 1);
        std::vector<char> buf(sbytes);
        std::ifstream f(statefile, std::ios::binary);
        if (!f || !f.read(buf.data(), (std::streamsize)sbytes)) {
            std::fprintf(stderr, "%s: ", kProg); std::fprintf(stderr, "cannot read %s\n", statefile);
            return 1;
        }
        if ((rc = fd23_set_state(s, buf.data(), sbytes, nt0))) return fail("restart state", rc);
    }
    if ((rc = fd23_run(s, nt, itrecord)) || (rc = fd23_sync(s))) return fail("run", rc);
    // seismograms
    const size_t cs = prec == FD23_F64 ? 8 : 4;
    const std::vector<int> *rx[2] = {&rxu, &rxw}, *rz[2] = {&rzu, &rzw};
    const char *suffix[2] = {kSH ? "_V" : "_U", "_W"};
    const float shiftx[2] = {kSH ? 0.0f : 0.5f, 0.0f}, shiftz[2] = {0.0f, -0.5f};
    for (int c = 0; c < (kSH ? 1 : 2); ++c) {
        const size_t ntr = rx[c]->size();
        int nrs = 0;
        if ((rc = fd23_get_seismograms(s, c, nullptr, 0, &nrs))) return fail("seismograms", rc);
        std::vector<unsigned char> raw((size_t)nrs * ntr * cs);
        if ((rc = fd23_get_seismograms(s, c, raw.data(), raw.size(), &nrs))) return fail("seismograms", rc);
        const std::string name = output + suffix[c];
        if (!write_file(name, raw.data(), raw.size())) {
            std::fprintf(stderr, "%s: ", kProg); std::fprintf(stderr, "cannot write %s\n", name.c_str());
            return 1;
        }
        const int ntrec = std::min(nrs, nt / itrecord);
        if (prec == FD23_F64) {
            // .db.isis: one 136-byte double header + double trace per receiver
            std::ofstream f(name + ".db.isis", std::ios::binary);
            std::vector<double> tr((size_t)ntrec);
            const double dshiftx[2] = {kSH ? 0.0 : 0.5, 0.0}, dshiftz[2] = {0.0, -0.5};
            for (size_t r = 0; r < ntr; ++r) {
                IsisTraceDb t;
                std::memset(&t, 0, sizeof t);
                const int ixr = (*rx[c])[r], izr = (*rz[c])[r];
                t.xr = (ixr + dshiftx[c]) * h;
                t.zr = (izr + dshiftz[c]) * h;
                t.xs = (double)(xs + src_shift_x) * h;
                t.zs = (double)(zs + src_shift_z) * h;
                t.nt = ntrec;
                t.samplerate = dt * (double)itrecord;
                t.gain = dt / h;
                t.ampstatic = 1.0;
                t.srcflagnum = xs;
                t.recflagnum = ixr;
                t.user[1] = usebox == 1 ? bw : 0;
                t.user[2] = 123456789;
                for (int k = 0; k < ntrec; ++k) tr[k] = reinterpret_cast<const double *>(raw.data())[(size_t)k * ntr + r];
                f.write((const char *)&t, sizeof t);
                f.write((const char *)tr.data(), (std::streamsize)(tr.size() * sizeof(double)));
            }
            if (!f) {
                std::fprintf(stderr, "%s: ", kProg); std::fprintf(stderr, "cannot write %s.db.isis\n", name.c_str());
                return 1;
            }
            continue;
        }
        // .isis: one header + trace per receiver, float samples
        std::ofstream f(name + ".isis", std::ios::binary);
        std::vector<float> tr((size_t)ntrec);
        for (size_t r = 0; r < ntr; ++r) {
            IsisTrace t;
            std::memset(&t, 0, sizeof t);
            const int ixr = (*rx[c])[r], izr = (*rz[c])[r];
            t.xr = ((float)ixr + shiftx[c]) * hf;
            t.zr = ((float)izr + shiftz[c]) * hf;
            t.xs = (float)xs * hf;
            t.zs = (float)zs * hf;
            t.nt = ntrec;
            t.samplerate = dtf * (float)itrecord;
            t.gain = dtf / hf;
            t.ampstatic = 1.0f;
            t.srcflagnum = xs;
            t.recflagnum = ixr;
            t.user[1] = t.user[2] = 123456789;
            for (int k = 0; k < ntrec; ++k) {
                const size_t o = (size_t)k * ntr + r;
                tr[k] = cs == 8 ? (float)reinterpret_cast<const double *>(raw.data())[o]
                                : reinterpret_cast<const float *>(raw.data())[o];
            }
            f.write((const char *)&t, sizeof t);
            f.write((const char *)tr.data(), (std::streamsize)(tr.size() * sizeof(float)));
        }
        if (!f) {
            std::fprintf(stderr, "%s: ", kProg); std::fprintf(stderr, "cannot write %s.isis\n", name.c_str());
            return 1;
        }
    }
    if (savestate) {
        std::snprintf(statefile, sizeof statefile, "state%06d", nt + nt0 - 1);
        std::vector<char> buf(sbytes);
        if ((rc = fd23_get_state(s, buf.data(), sbytes))) return fail("state", rc);
        if (!write_file(statefile, buf.data(), sbytes)) {
            std::fprintf(stderr, "%s: ", kProg); std::fprintf(stderr, "cannot write %s\n", statefile);
            return 1;
        }
    }
    fd23_destroy(s);
    std::printf("finish\n");
    return 0;
}
