// Model and station input (host only): the reference's .mdl polygon models,
// raster models and station files.
//
// .mdl (PD/model/model.cpp:240-369): one command per line -- "DEF name x z"
// names a vertex, "BACK vp vs den" sets the background, "POLY vp vs den"
// starts a polygon whose vertices follow on lines that begin with a tab
// (coordinate pairs, or vertex names when the line's first token is a name).
// A negative vs or den is a factor of vp.  Lines that are empty or start
// with '#' are skipped.  Rasterising (get_elas_model, model.cpp:175-232):
// the background everywhere, then each polygon in file order over the cells
// of its bounding box (widened by one cell) whose point (ix*h, iz*h) is
// inside it (crossing-number test; points on an edge count as inside), so a
// later polygon wins where polygons overlap.
//
// Raster models (PD/model/util.cpp:12-22): <name>.vp, <name>.vs, <name>.den,
// nx*nz float32 each, x fastest.
//
// Station files (PD/record/cu_record.cu:30-76): one station per line, "z x".
#include <algorithm>
#include <cctype>
#include <cstdlib>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include "fd23_internal.h"

namespace {

struct Poly {
    double vp, vs, den;
    std::vector<double> x, z;
};

bool inside(double xp, double zp, const Poly &p)
{
    const int n = (int)p.x.size();
    int nleft = 0;
    double x2 = p.x[n - 1], z2 = p.z[n - 1];
    for (int j = 0; j < n; ++j) {
        const double x1 = x2, z1 = z2;
        x2 = p.x[j];
        z2 = p.z[j];
        const double zlo = z1 < z2 ? z1 : z2, zhi = z1 > z2 ? z1 : z2;
        if (zlo >= zp || zhi < zp) continue;
        if (z1 == z2) {  // horizontal edge at the query depth
            const double xlo = x1 < x2 ? x1 : x2, xhi = x1 > x2 ? x1 : x2;
            if (xp > xhi) continue;
            if (xp >= xlo) return true;
            ++nleft;
            continue;
        }
        const double xi = x1 + (zp - z1) * (x2 - x1) / (z2 - z1);
        if (xi == xp) return true;
        if (xi > xp) ++nleft;
    }
    return nleft % 2 == 1;
}

std::vector<std::string> tokens(const std::string &line)
{
    std::vector<std::string> t;
    std::istringstream is(line);
    std::string w;
    while (is >> w) t.push_back(w);
    return t;
}

int parse_mdl(const char *path, std::vector<Poly> &polys)
{
    std::ifstream f(path);
    if (!f) return FD23_ERR_ARG;
    std::vector<std::string> lines;
    for (std::string l; std::getline(f, l);) {
        if (!l.empty() && l.back() == '\r') l.pop_back();
        lines.push_back(l);
    }
    std::map<std::string, std::pair<double, double>> defs;
    Poly back{};
    bool have_back = false;
    std::vector<Poly> rest;
    for (size_t k = 0; k < lines.size();) {
        const std::string line = lines[k++];
        if (line.empty() || line[0] == '#') continue;
        std::vector<std::string> a = tokens(line);
        if (a.empty()) continue;
        std::string key = a[0];
        for (auto &c : key) c = (char)std::toupper((unsigned char)c);
        if (key == "DEF") {
            if (a.size() != 4) return FD23_ERR_ARG;
            defs[a[1]] = {std::atof(a[2].c_str()), std::atof(a[3].c_str())};
            continue;
        }
        if (key != "BACK" && key != "POLY") return FD23_ERR_ARG;
        if (a.size() != 4) return FD23_ERR_ARG;
        Poly p{};
        p.vp = std::atof(a[1].c_str());
        p.vs = std::atof(a[2].c_str());
        p.den = std::atof(a[3].c_str());
        if (p.vs < 0.0) p.vs = -p.vp * p.vs;
        if (p.den < 0.0) p.den = -p.vp * p.den;
        if (key == "BACK") {
            back = p;
            have_back = true;
            continue;
        }
        while (k < lines.size() && !lines[k].empty() && lines[k][0] == '\t') {
            std::vector<std::string> v = tokens(lines[k++]);
            if (v.empty()) continue;
            const bool names = std::isalpha((unsigned char)v[0][0]) != 0;
            for (size_t i = 0; i < v.size(); ++i) {
                if (names) {
                    auto it = defs.find(v[i]);
                    if (it == defs.end()) return FD23_ERR_ARG;
                    p.x.push_back(it->second.first);
                    p.z.push_back(it->second.second);
                } else {
                    if (i + 1 >= v.size()) return FD23_ERR_ARG;
                    p.x.push_back(std::atof(v[i].c_str()));
                    p.z.push_back(std::atof(v[i + 1].c_str()));
                    ++i;
                }
            }
        }
        if (p.x.size() < 3) return FD23_ERR_ARG;
        rest.push_back(p);
    }
    if (!have_back) return FD23_ERR_ARG;
    polys.clear();
    polys.push_back(back);
    polys.insert(polys.end(), rest.begin(), rest.end());
    return FD23_OK;
}

int clampi(int v, int hi) { return v < 0 ? 0 : (v > hi ? hi : v); }

void rasterise(const std::vector<Poly> &polys, int nx, int nz, double h, double *vp, double *vs, double *den)
{
    const size_t n = (size_t)nx * nz;
    for (size_t k = 0; k < n; ++k) {
        vp[k] = polys[0].vp;
        vs[k] = polys[0].vs;
        den[k] = polys[0].den;
    }
    for (size_t p = 1; p < polys.size(); ++p) {
        const Poly &q = polys[p];
        double x1 = 1e28, x2 = -1e28, z1 = 1e28, z2 = -1e28;
        for (size_t j = 0; j < q.x.size(); ++j) {
            x1 = std::min(x1, q.x[j]);
            x2 = std::max(x2, q.x[j]);
            z1 = std::min(z1, q.z[j]);
            z2 = std::max(z2, q.z[j]);
        }
        const int ix1 = clampi((int)(x1 / h - 1), nx - 1), ix2 = clampi((int)(x2 / h + 1), nx - 1);
        const int iz1 = clampi((int)(z1 / h - 1), nz - 1), iz2 = clampi((int)(z2 / h + 1), nz - 1);
        for (int iz = iz1; iz <= iz2; ++iz)
            for (int ix = ix1; ix <= ix2; ++ix)
                if (inside(h * (double)ix, h * (double)iz, q)) {
                    const size_t k = (size_t)iz * nx + ix;
                    vp[k] = q.vp;
                    vs[k] = q.vs;
                    den[k] = q.den;
                }
    }
}

bool ends_with(const std::string &s, const std::string &e)
{
    return s.size() > e.size() && s.compare(s.size() - e.size(), e.size(), e) == 0;
}

}  // namespace

extern "C" {

int fd23_read_model(const char *name, int nx, int nz, double h, double *vp, double *vs, double *den)
{
    if (!name || nx < 1 || nz < 1 || !(h > 0) || !vp || !vs || !den) return FD23_ERR_ARG;
    const std::string s(name);
    if (ends_with(s, ".mdl")) {
        std::vector<Poly> polys;
        const int rc = parse_mdl(name, polys);
        if (rc) return rc;
        rasterise(polys, nx, nz, h, vp, vs, den);
        return FD23_OK;
    }
    const size_t n = (size_t)nx * nz;
    std::vector<float> buf(n);
    double *out[3] = {vp, vs, den};
    const char *ext[3] = {"vp", "vs", "den"};
    for (int q = 0; q < 3; ++q) {
        std::ifstream f(s + "." + ext[q], std::ios::binary);
        if (!f.read(reinterpret_cast<char *>(buf.data()), (std::streamsize)(n * sizeof(float)))) return FD23_ERR_ARG;
        for (size_t k = 0; k < n; ++k) out[q][k] = buf[k];
    }
    return FD23_OK;
}

int fd23_read_stations(const char *path, int *rx, int *rz, int cap)
{
    if (!path || cap < 0 || (cap > 0 && (!rx || !rz))) return FD23_ERR_ARG;
    std::ifstream f(path);
    if (!f) return FD23_ERR_ARG;
    int n = 0;
    long long z, x;
    while (f >> z >> x) {
        if (2 * n + 2 <= cap) {
            rx[2 * n] = (int)x;
            rz[2 * n] = (int)z;
            rx[2 * n + 1] = (int)x - 1;
            rz[2 * n + 1] = (int)z;
        } else if (cap > 0) {
            return FD23_ERR_ARG;
        }
        ++n;
    }
    return 2 * n;
}

}  // extern "C"
