// Reference set-up and host-step harness -- TEST INFRASTRUCTURE ONLY.
//
// Drives the reference programs' own host code, compiled from their sources
// where they lie by oracle/build_ref.py, on inputs the fixture generator
// (tests/golden/make_ref_pins.py) writes, and dumps what that code computes,
// so the oracle's restatements can be pinned to it.  One source, three
// programs (built with the matching program root on the include path):
//
//   REF_PN  PSV/clean_nobox, the FP32 P-SV program: MATERIAL::get_model
//           (material/material.cpp) and CPML::CPML (cpml/cpml.cpp) in float.
//   REF_SH  SH, the FP32 SH program: MATERIAL::get_model, CPML::CPML, and
//           one host step (fd/fd.cpp step_stress, step_velocity) from a
//           state the caller gives.
//   REF_PD  PSV/psv_clean_double, the FP64 P-SV program: MATERIAL::get_model,
//           CPML::CPML, BOX::init_box (box/box.cpp: ring lists, the box
//           material from MATERIAL::init_for_box_from_full), BOX::setboxsource
//           over the frames of a displacement-plane file, and the residual
//           updates step_stress_r / step_velocity_r (fd/fd.cpp) from a
//           residual field the caller gives.
//
// Usage: harness <nx> <nz> <h> <dt> <npml> <pml_dt> <pml_r> <pml_v> <pml_fc>
//                <model prefix> <out> [REF_SH: <state in>]
//                [REF_PD: <xs> <zs> <bw> <srcpvel> <srcsvel> <srcden>
//                         <planes file> <frames> <residual in>]
// The model rasters are <prefix>.vp / .vs / .den (float, nx*nz, row-major),
// as the reference's read_model reads them.  Output: raw arrays in the
// program's precision, in the order written below.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "cpml/cpml.h"
#include "material/material.h"
#include "param/param.h"
#if defined(REF_SH) || defined(REF_PD)
#include "fd/fd.h"
#include "field/field.h"
#endif
#if defined(REF_PD)
#include "box/box.h"
#endif

#if defined(REF_PD)
typedef double real;
#else
typedef float real;
#endif

static void put(FILE *f, const real *p, size_t n) { fwrite(p, sizeof(real), n, f); }
static void put_i(FILE *f, const int *p, size_t n) { fwrite(p, sizeof(int), n, f); }
static bool get(const char *name, real *p, size_t n)
{
    FILE *f = fopen(name, "rb");
    if (!f) return false;
    const bool ok = fread(p, sizeof(real), n, f) == n;
    fclose(f);
    return ok;
}

int main(int argc, char **argv)
{
#if defined(REF_PD)
    const int need = 21;
#elif defined(REF_SH)
    const int need = 13;
#else
    const int need = 12;
#endif
    if (argc < need) {
        fprintf(stderr, "usage: see oracle/ref_setup_harness.cpp\n");
        return 2;
    }
    static PARAM p;
    memset(&p, 0, sizeof p);
    p.nx = atoi(argv[1]);
    p.nz = atoi(argv[2]);
    p.h = atof(argv[3]);
    p.dt = atof(argv[4]);
    p.npml = atoi(argv[5]);
    p.pml_dt = atof(argv[6]);
    p.pml_r = atof(argv[7]);
    p.pml_v = atof(argv[8]);
    p.pml_fc = atof(argv[9]);
    strncpy(p.modelname, argv[10], sizeof p.modelname - 1);
#if defined(REF_PD)
    // the box parameters first: MATERIAL::init_for_full copies the source
    // material (srcpvel, srcsvel, srcden) that init_for_box_from_full uses
    p.xs = atoi(argv[12]);
    p.zs = atoi(argv[13]);
    p.bw = atoi(argv[14]);
    p.srcpvel = atof(argv[15]);
    p.srcsvel = atof(argv[16]);
    p.srcden = atof(argv[17]);
    strncpy(p.sourcefile, argv[18], sizeof p.sourcefile - 1);
    const int frames = atoi(argv[19]);
    p.usebox = 1;
#endif
    const int nx = p.nx, nz = p.nz;
    const size_t n = (size_t)nx * nz;
    FILE *out = fopen(argv[11], "wb");
    if (!out) return 3;

    MATERIAL mat;
    mat.init_for_full(p);
    mat.get_model(p);
    CPML cpml(p);
#if defined(REF_SH)
    put(out, mat.MUX, n);
    put(out, mat.MUZ, n);
    put(out, mat.BV, n);
    // b, c, k of Tx_x V_x (nx) Tz_z V_z (nz)
    const PMLVARIABLE *v[3] = {&cpml.b, &cpml.c, &cpml.k};
    for (int q = 0; q < 3; ++q) {
        put(out, v[q]->Tx_x, nx);
        put(out, v[q]->V_x, nx);
        put(out, v[q]->Tz_z, nz);
        put(out, v[q]->V_z, nz);
    }
    // one host step from the given state [V, Tx, Tz] (memory variables zero)
    FIELD fld;
    fld.nx = nx;
    fld.nz = nz;
    std::vector<real> st(3 * n);
    if (!get(argv[12], st.data(), st.size())) return 4;
    fld.V = st.data();
    fld.Tx = st.data() + n;
    fld.Tz = st.data() + 2 * n;
    step_stress(fld, mat, cpml);
    step_velocity(fld, mat, cpml);
    put(out, st.data(), st.size());
#else
    put(out, mat.LAM, n);
    put(out, mat.MU, n);
    put(out, mat.MUA, n);
    put(out, mat.BU, n);
    put(out, mat.BW, n);
    // b, c, k of Txx_x Txz_x U_x W_x (nx) Tzz_z Txz_z U_z W_z (nz)
    const PMLVARIABLE *v[3] = {&cpml.b, &cpml.c, &cpml.k};
    for (int q = 0; q < 3; ++q) {
        put(out, v[q]->Txx_x, nx);
        put(out, v[q]->Txz_x, nx);
        put(out, v[q]->U_x, nx);
        put(out, v[q]->W_x, nx);
        put(out, v[q]->Tzz_z, nz);
        put(out, v[q]->Txz_z, nz);
        put(out, v[q]->U_z, nz);
        put(out, v[q]->W_z, nz);
    }
#endif
#if defined(REF_PD)
    BOX box;
    box.init_box(p, mat);
    const int bw = box.bw;
    const size_t nb = (size_t)bw * bw;
    const int head[4] = {box.n_sub, box.n_add, box.start_x, box.start_z};
    put_i(out, head, 4);
    put_i(out, box.r_sub_idx, box.n_sub);
    put_i(out, box.a_sub_idx, box.n_sub);
    put_i(out, box.r_add_idx, box.n_add);
    put_i(out, box.a_add_idx, box.n_add);
    put(out, box.p_bmat->LAM, nb);
    put(out, box.p_bmat->MU, nb);
    put(out, box.p_bmat->MUA, nb);
    put(out, box.p_bmat->BU, nb);
    put(out, box.p_bmat->BW, nb);
    // incident field of frames 1 .. frames-1 (each from frames k-1 and k)
    for (int k = 1; k < frames; ++k) {
        box.setboxsource();
        put(out, box.p_sfield->U, nb);
        put(out, box.p_sfield->W, nb);
        put(out, box.p_sfield->Txx, nb);
        put(out, box.p_sfield->Txz, nb);
        put(out, box.p_sfield->Tzz, nb);
    }
    // residual updates on the given bw x bw residual field [U W Txx Txz Tzz]
    FIELD r;
    memset(&r, 0, sizeof r);
    r.nx = bw;
    r.nz = bw;
    std::vector<real> rs(5 * nb);
    if (!get(argv[20], rs.data(), rs.size())) return 4;
    r.U = rs.data();
    r.W = rs.data() + nb;
    r.Txx = rs.data() + 2 * nb;
    r.Txz = rs.data() + 3 * nb;
    r.Tzz = rs.data() + 4 * nb;
    step_stress_r(r, *box.p_bmat);
    step_velocity_r(r, *box.p_bmat);
    put(out, rs.data(), rs.size());
#endif
    fclose(out);
    return 0;
}
