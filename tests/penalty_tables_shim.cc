// C entry points over the product's divcurl table builders
// (mia_gb300/csrc/tables.cc), compiled by tests/test_penalty_tables.py
// together with tables.cc so that the CPU tests can compare the tables with
// the oracle's without a GPU.
#include <cstddef>
#include <vector>

#include "../mia_gb300/csrc/tables.hh"

extern "C" void shim_penalty3(const int csize[3], const float range[3], double wdiv, double wrot, double *out)
{
    const std::vector<double> P = mgr::penalty3_cells(csize, range, wdiv, wrot);
    for (size_t k = 0; k < P.size(); ++k) out[k] = P[k];
}

extern "C" size_t shim_penalty2(const int csize[2], const float range[2], double wd, double wr, int *rowptr,
                                int *col, double *val, size_t cap)
{
    std::vector<int> rp, cl;
    std::vector<double> v;
    mgr::penalty2_cells(csize, range, wd, wr, rp, cl, v);
    for (size_t k = 0; k < rp.size(); ++k) rowptr[k] = rp[k];
    for (size_t k = 0; k < cl.size() && k < cap; ++k) {
        col[k] = cl[k];
        val[3 * k] = v[3 * k];
        val[3 * k + 1] = v[3 * k + 1];
        val[3 * k + 2] = v[3 * k + 2];
    }
    return cl.size();
}
