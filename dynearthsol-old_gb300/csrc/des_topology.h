// Library-internal entry of the host topology build (topology.cpp).
#pragma once

#include "des_gpu.h"

namespace des {

// des_topology_build with the support lists left out when !support (the
// device state builds its own, des_support.cuh); the support pointers of the
// result are then NULL.
int topology_build(const des_mesh_view *m, des_topology **out, bool support);

}  // namespace des
