// ps_coupling.h -- library-internal link between the LBM and LSM handles
// (fluid wall load -> lattice-spring load).
#pragma once

namespace ps {

// Wall load (S1:3849-3882, with the given rsi) of the lattice's current
// state on the periodic corner-node box, as three planes [3][nx*ny*nz] in
// device memory owned by the lattice (valid until its next wall-load call
// or its destruction).  Synchronises the lattice's stream before returning.
int lbm_wall_load_box(void* lattice, double rsi, const double** d_box, int dims[3]);

}  // namespace ps
