// tune.cc — the table of tuned tile shapes.  mia_gb300/autotune.py times
// every compiled tile shape of the split path on the target GPU for a set
// of image sizes, spline rates and costs, and commits the fastest shape of
// each case to mia_gb300/tiles.json; the build writes that table into
// tile_table.inc (one {dim, spacing, voxels, {tx, ty, tz}} line per case).
#include "tune.hh"

#include <cmath>

namespace mgr {

namespace {

struct TileEntry {
    int dim;
    double spacing;   // mean voxels per coefficient interval
    double voxels;
    int tile[3];
};

const TileEntry k_table[] = {
#include "tile_table.inc"
    {0, 0.0, 0.0, {0, 0, 0}},   // end of the table
};

}  // namespace

bool tuned_tile(int dim, const int n[3], const int nc[3], int tile[3])
{
    double sp = 0.0, vox = 1.0;
    for (int k = 0; k < dim; ++k) {
        sp += double(n[k] - 1) / double(nc[k] > 4 ? nc[k] - 3 : 1);
        vox *= double(n[k]);
    }
    sp /= dim;
    int best = -1;
    double bd = 0.0;
    for (int i = 0; k_table[i].dim != 0; ++i) {
        const TileEntry &e = k_table[i];
        if (e.dim != dim) continue;
        const double d = std::fabs(std::log(e.spacing / sp)) + 0.5 * std::fabs(std::log(e.voxels / vox));
        if (best < 0 || d < bd) {
            best = i;
            bd = d;
        }
    }
    if (best < 0) return false;
    for (int k = 0; k < 3; ++k) tile[k] = k_table[best].tile[k];
    return true;
}

}  // namespace mgr
