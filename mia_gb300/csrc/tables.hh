// tables.hh — host-side per-level tables (see tables.cc).
#pragma once

#include <memory>
#include <vector>

namespace mgr {

struct AxisHost {
    int n = 0, nc = 0, t = 0, nt = 0, fc = 0, ac = 0;
    float scale = 0.0f;
    std::vector<int> fs;       // n
    std::vector<float> fw;     // n x 4
    std::vector<int> as;       // n
    std::vector<float> aw;     // n x 4
    std::vector<int> rows;     // nc x (first, len)
    std::vector<int> ftile0;   // nt
    std::vector<int> atile0;   // nt
    std::vector<int> gtile;    // nc x (lo, hi)
    std::vector<int> glist;    // 3D: nc x GATHER_LMAX partial-slot offset parts
    std::vector<int> glen;     // 3D: nc list lengths (-1: too long)
};

int csize_from_rate(int size, float rate);
void build_axis(AxisHost &ax, int n, int nc, int tile);
// divcurl penalty tables (see tables.cc).  3D: the 9^3 cells of offsets
// d = i - j (index ((dz + 4) 9 + dy + 4) 9 + dx + 4), six entries each
// (xx, xy, yy, yz, zz, xz).  2D: per coefficient i (row, CSR) the
// coefficients j it couples with, three entries each (xx, yy, xy).
std::vector<double> penalty3_cells(const int csize[3], const float range[3], double wdiv, double wrot);
void penalty2_cells(const int csize[2], const float range[2], double wd, double wr, std::vector<int> &rowptr,
                    std::vector<int> &col, std::vector<double> &val);
// the same rounded to float for the device; 2D cells padded to four floats
std::vector<float> build_penalty3(const int csize[3], const float range[3], double wdiv, double wrot);
void build_penalty2(const int csize[2], const float range[2], double wd, double wr, std::vector<int> &rowptr,
                    std::vector<int> &col, std::vector<float> &val);

// build_penalty2 through a process-wide cache keyed by (csize, range, wd,
// wr): the frames of a series share their grid, so each table is built once
struct Penalty2Table {
    std::vector<int> rowptr, col;
    std::vector<float> val;
};
std::shared_ptr<const Penalty2Table> penalty2_cached(const int csize[2], const float range[2], double wd, double wr);

}  // namespace mgr
