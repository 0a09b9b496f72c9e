// Material table (host side): the reference's mktable (PD/material/
// mktable.cpp:43-106, called by SH/main.cpp:154) on the GB300 layout.
//
// The reference stores an int index per cell and a table of the distinct
// (BU, BW, MU, MUA, LAM) tuples, found by comparing each cell's tuple with the
// last 10000 entries, and gives up past nx*nz/100 entries.  Here every
// cell's tuple of storage values (the dt/h-scaled material as the sweep reads
// it, in the solver's storage type) is matched exactly, bit for bit, so a
// lookup returns the very value the material array holds; the index is one
// byte in the padded layout (entry 0 = the zero tuple of the padding), which
// caps the table at 256 entries.  The sweep's material traffic drops from
// 5 (P-SV) or 3 (SH) values per cell to one byte.
#include <cuda_runtime.h>

#include <cstring>
#include <string>
#include <unordered_map>
#include <vector>

#include "fd23_solver.h"

namespace fd23 {

void free_material_table(fd23_solver *s)
{
    cudaFree(s->d_midx);
    cudaFree(s->d_mtab);
    s->d_midx = nullptr;
    s->d_mtab = nullptr;
    s->table_n = 0;
}

int build_material_table(fd23_solver *s)
{
    const size_t n = (size_t)s->d.nx * s->d.nz, es = s->es;
    const int nm = s->nmat;
    std::vector<unsigned char> mat((size_t)nm * n * es);
    for (int m = 0; m < nm; ++m) {
        const int rc = download_grid(s, s->mat[m], mat.data() + (size_t)m * n * es, es);
        if (rc) return rc;
    }
    CK(cudaStreamSynchronize(s->stream));
    // tuples as byte strings, entry 0 the zero tuple
    std::unordered_map<std::string, int> seen;
    std::vector<std::string> entries;
    std::string key(nm * es, '\0');
    seen.emplace(key, 0);
    entries.push_back(key);
    const Layout &L = s->L;
    std::vector<unsigned char> idx(L.elems(), 0);
    for (int iz = 0; iz < s->d.nz; ++iz)
        for (int ix = 0; ix < s->d.nx; ++ix) {
            const size_t c = (size_t)iz * s->d.nx + ix;
            for (int m = 0; m < nm; ++m) std::memcpy(&key[m * es], mat.data() + ((size_t)m * n + c) * es, es);
            auto it = seen.find(key);
            int e;
            if (it != seen.end()) {
                e = it->second;
            } else {
                if ((int)entries.size() >= kTabEntries) return FD23_ERR_UNSUPPORTED;
                e = (int)entries.size();
                seen.emplace(key, e);
                entries.push_back(key);
            }
            idx[(size_t)L.origin + (size_t)iz * L.pitch + ix] = (unsigned char)e;
        }
    std::vector<unsigned char> tab((size_t)nm * kTabEntries * es, 0);
    for (size_t e = 0; e < entries.size(); ++e)
        for (int m = 0; m < nm; ++m)
            std::memcpy(tab.data() + ((size_t)m * kTabEntries + e) * es, &entries[e][m * es], es);
    if (!s->d_midx) {
        int rc = dev_alloc((void **)&s->d_midx, L.elems());
        if (!rc) rc = dev_alloc(&s->d_mtab, tab.size());
        if (rc) {
            free_material_table(s);
            return rc;
        }
    }
    CK(cudaMemcpy(s->d_midx, idx.data(), idx.size(), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(s->d_mtab, tab.data(), tab.size(), cudaMemcpyHostToDevice));
    s->table_n = (int)entries.size();
    return s->fused ? encode_maps(s) : FD23_OK;
}

}  // namespace fd23

using namespace fd23;

extern "C" {

int fd23_set_material_table(fd23_solver *s, int on)
{
    if (!s) return FD23_ERR_ARG;
    CK(cudaSetDevice(s->d.device));
    CK(cudaStreamSynchronize(s->stream));
    if (!on) {
        free_material_table(s);
        s->table_on = false;
        return s->fused ? encode_maps(s) : FD23_OK;
    }
    if (!s->have_material) return FD23_ERR_ORDER;
    if (s->box_on) return FD23_ERR_UNSUPPORTED;
    const int rc = build_material_table(s);
    if (rc) {
        free_material_table(s);
        s->table_on = false;
        if (s->fused) encode_maps(s);
        return rc;
    }
    s->table_on = true;
    return s->table_n;
}

}  // extern "C"
