// Glue between the reference's Param / Variables (parameters.hpp) and the C
// ABI of libdes_gb300.so.  Compiled inside the reference's build, against its
// headers; see INTEGRATION.md.
#pragma once

#include "des_gpu.h"

struct Param;
struct Variables;

// Creates the device state for var's mesh and uploads the loop state (call
// after init() or restart(), and again after every remesh).  Returns NULL and
// prints the reason when the library rejects the configuration.
des_gpu *des_shim_attach(const Param &param, Variables &var);

// Replaces the loop body dynearthsol.cxx:358-394 for nsteps iterations; var's
// time, dt and steps are updated, the arrays stay on the device.  Returns the
// library's status code; 11 where the reference would exit(11).
int des_shim_step(des_gpu *g, Variables &var, int nsteps);

// Copies device fields back into var's arrays before output, checkpoint or
// remesh (mask: DES_F_* bits, DES_F_ALL for everything).
int des_shim_download(des_gpu *g, Variables &var, unsigned mask);
