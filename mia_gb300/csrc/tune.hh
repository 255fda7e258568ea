// tune.hh — the tile shapes chosen by the autotuner (see tune.cc).
#pragma once

namespace mgr {

// The tuned tile for a level of image size n with coefficient grid nc: the
// tile of the autotuner's case nearest in mean coefficient spacing and in
// image size (log scale), of the same dimension.  False when the table has
// no case of this dimension.
bool tuned_tile(int dim, const int n[3], const int nc[3], int tile[3]);

}  // namespace mgr
