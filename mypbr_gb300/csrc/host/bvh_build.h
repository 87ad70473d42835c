// Host-side binned-SAH BVH build over the flat scene's primitives.
#pragma once

#include <vector>

#include "../../../include/mypbr_gpu.h"
#include "host_math.h"

namespace mypbr_host {

struct BuildItem {
    Box box;
    V3 centroid;
    mypbr_prim_ref ref;
};

// Builds the tree over items (reordered internally) into nodes / prims in the
// reference's depth-first layout. An empty item list gives one empty leaf.
void build_bvh(std::vector<BuildItem> items, std::vector<mypbr_bvh_node>& nodes, std::vector<mypbr_prim_ref>& prims);

// The Kulla-Conty E(mu, alpha) table and E_avg (1056 doubles).
void ggx_albedo_table(double* out);

}  // namespace mypbr_host
