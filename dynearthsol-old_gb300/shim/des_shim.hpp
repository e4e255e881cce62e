// Glue between the reference's Param / Variables (parameters.hpp) and the C
// ABI of libdes_gb300.so.  Compiled inside the reference's build, against its
// headers.
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

// After phase_changes (phasechanges.cxx:232-258) at steps % 10 == 0: the
// device takes var.elemmarkers and recomputes dt as compute_dt does right
// after it (dynearthsol.cxx:382-393); var.dt is updated.
int des_shim_phase_changes(des_gpu *g, const Param &param, Variables &var);

// After the reference's remesh (remeshing.cxx:1963-2067) has run on var's
// host arrays (download them first): the device takes the new mesh, the
// interpolated fields and the remapped markers, and repeats remesh's
// compute_volume / compute_mass / compute_shape_fn / coord0 reset.
int des_shim_remeshed(des_gpu *g, const Param &param, Variables &var);
