// grid_refine.cuh -- regular refinement of unstructured levels on the device.
#pragma once

#include "common.cuh"

namespace ug4gb {

typedef unsigned long long u64;

// The objects of the Dirichlet subsets a level carries to its refinement.
struct DevDir {
    DevBuf<u64> edges;               // sorted unique (a << 32 | b), a < b
    int n_edges = 0;
    DevBuf<int4> faces;              // cyclic corners (w = -1: triangle), unique by corner set
    int n_faces = 0;
    DevBuf<unsigned char> edir;      // elements of Dirichlet subsets
};

// F = one regular refinement of the unstructured level C: coordinates,
// elements, Dirichlet vertices and parents (colourings are left to the
// caller); Fd = the Dirichlet objects of F.
void refine_device(Ctx &c, const Level &C, const DevDir &Cd, Level &F, DevDir &Fd);

}  // namespace ug4gb
