/*
 * des_gpu.h -- C ABI of the GB300 (sm_103a) time-step library for the
 * DynEarthSol3D explicit loop (dynearthsol.cxx:354-394).
 *
 * Every pointer in these structs is a plain host pointer into storage laid out
 * exactly like the reference's Array2D<T,N> (array2d.hpp:86-87: row i starts at
 * a_ + N*i) or std::vector<double>; the library keeps its own structure-of-arrays
 * copies in device memory.  No torch or CUDA type appears in any signature.
 *
 * Threading: one handle is used by one host thread.  Calls are ordered on the
 * handle's private CUDA stream; des_gpu_download, des_gpu_step (when it fills a
 * report) and des_gpu_compute_dt synchronise that stream before returning.
 *
 * Errors: every entry point returns 0 (DES_OK) or one of the DES_ERR_* codes.
 * Where the reference calls std::exit(code) the library returns the same code
 * (11 for "dt <= 0", geometry.cxx:321-325; 12 for inconsistent topology,
 * mesh.cxx:1676-1678 and matprops.cxx:516-518; 1 for an unknown rheology or
 * option, rheology.cxx:641-644, fields.cxx:302-304).
 */
#ifndef DES_GPU_H
#define DES_GPU_H

#ifdef __cplusplus
extern "C" {
#endif

#define DES_MAX_MAT 16
#define DES_NBDRY   10   /* constants.hpp:37 nbdrytypes */

/* return codes */
#define DES_OK              0
#define DES_ERR_OPTION      1   /* unknown rheology / damping / surface option */
#define DES_ERR_ARG         2   /* bad pointer, size or mask */
#define DES_ERR_CUDA        3   /* a CUDA runtime call failed */
#define DES_ERR_NOMEM       4   /* device allocation failed */
#define DES_ERR_UNSUPPORTED 5   /* 2D / plane strain / closure preconditions */
#define DES_ERR_SIZE        6   /* size above a fixed limit of the entry point */
#define DES_ERR_DT         11   /* dt <= 0 (geometry.cxx:321-325) or NaN/Inf coordinates (output.cxx:195-208) */
#define DES_ERR_TOPOLOGY   12   /* a segment is on no element (mesh.cxx:1676-1678) */

/* status bits reported by des_gpu_step (device-side status word) */
#define DES_STATUS_DT_NONPOSITIVE 0x1u   /* compute_dt gave dt <= 0 */
#define DES_STATUS_NONFINITE      0x2u   /* NaN/Inf in the coordinates (output.cxx:195-208) */
#define DES_STATUS_NEG_VOLUME     0x4u   /* an element volume became <= 0 */
#define DES_STATUS_QL_NOCONV      0x8u   /* QL eigen fallback did not converge in 30 sweeps */

/* rheology codes (matprops.hpp:124-130) */
#define DES_RH_ELASTIC 1
#define DES_RH_VISCOUS 2
#define DES_RH_PLASTIC 4
#define DES_RH_MAXWELL 3
#define DES_RH_EP      5
#define DES_RH_EVP     7

/* arithmetic form of the step */
#define DES_PREC_FP64 0   /* plain FP64, parity with the reference functions */
#define DES_PREC_FP32 1   /* FP32 element arithmetic, FP64 coordinates/volumes/shape
                             derivatives/plastic strain/temperature/dt */

/* field mask for upload / download */
#define DES_F_COORD        (1u << 0)
#define DES_F_VEL          (1u << 1)
#define DES_F_FORCE        (1u << 2)
#define DES_F_TEMPERATURE  (1u << 3)
#define DES_F_MASS         (1u << 4)   /* mass, tmass, volume_n */
#define DES_F_NTMP         (1u << 5)
#define DES_F_VOLUME       (1u << 6)   /* volume, volume_old */
#define DES_F_STRESS       (1u << 7)
#define DES_F_STRAIN       (1u << 8)
#define DES_F_STRAIN_RATE  (1u << 9)
#define DES_F_PLSTRAIN     (1u << 10)  /* plstrain, delta_plstrain */
#define DES_F_DPRESSURE    (1u << 11)
#define DES_F_EDVOLDT      (1u << 12)
#define DES_F_SHAPE        (1u << 13)  /* shpdx, shpdy, shpdz */
#define DES_F_TMP_RESULT   (1u << 14)  /* tmp_result, tmp_result_sg */
#define DES_F_SCALARS      (1u << 15)  /* time, dt, steps */
#define DES_F_COORD0       (1u << 16)
#define DES_F_ALL          0x1ffffu
/* what one step of the loop reads or writes (the state a drop-in keeps on the host) */
#define DES_F_STEP_STATE   (DES_F_COORD | DES_F_VEL | DES_F_FORCE | DES_F_TEMPERATURE | \
                            DES_F_MASS | DES_F_NTMP | DES_F_VOLUME | DES_F_STRESS |       \
                            DES_F_STRAIN | DES_F_STRAIN_RATE | DES_F_PLSTRAIN |           \
                            DES_F_DPRESSURE | DES_F_EDVOLDT | DES_F_SHAPE | DES_F_SCALARS)

/* One material property vector of Param::mat (parameters.hpp:187-205).
 * len is 1 (one value for all materials) or nmat, exactly as the reference's
 * VectorBase::create accepts (matprops.cxx:509-520); the two lengths give
 * different averaging (matprops.cxx:436-461). */
typedef struct des_matvec {
    int    len;
    double v[DES_MAX_MAT];
} des_matvec;

/* The Param and Variables scalars the hot path reads (parameters.hpp:82-206,
 * 245-256). */
typedef struct des_params {
    /* Control */
    double gravity;
    double inertial_scaling;
    double dt_fraction;
    double fixed_dt;
    double damping_factor;
    double surface_diffusivity;   /* surface_process_option 1 (bc.cxx:598-730) */
    int    damping_option;
    int    ref_pressure_option;
    int    surface_process_option;
    int    is_quasi_static;
    int    has_thermal_diffusion;
    /* BC */
    double surface_temperature;
    double winkler_delta_rho;
    double elastic_foundation_constant;
    int    has_winkler_foundation;
    int    has_elastic_foundation;
    int    has_water_loading;
    /* Mesh */
    double zlength;
    /* Mat */
    int    rheol_type;
    int    nmat;
    int    is_plane_strain;
    double visc_min, visc_max, tension_max, therm_diff_max;
    des_matvec rho0, alpha, bulk_modulus, shear_modulus;
    des_matvec visc_exponent, visc_coefficient, visc_activation_energy;
    des_matvec heat_capacity, therm_cond;
    des_matvec pls0, pls1, cohesion0, cohesion1;
    des_matvec friction_angle0, friction_angle1, dilation_angle0, dilation_angle1;
    /* Variables (set by init_var / create_boundary_normals) */
    int    vbc_types[DES_NBDRY];
    double vbc_values[DES_NBDRY];
    double max_vbc_val;
    double compensation_pressure;
    double bnormals[DES_NBDRY][3];
    double edge_vectors[DES_NBDRY][DES_NBDRY][3];   /* [i][j], i < j */
    /* library options */
    int    precision;           /* DES_PREC_* */
} des_params;

/* Mesh as the reference holds it after create_new_mesh (parameters.hpp:258-263). */
typedef struct des_mesh_view {
    int nnode, nelem, nseg, nmat;
    const int *connectivity;   /* [nelem][4]  conn_t */
    const int *segment;        /* [nseg][3]   segment_t */
    const int *segflag;        /* [nseg]      segflag_t */
    const int *elemmarkers;    /* [nelem][nmat] rows of int_vec2D (marker counts per material) */
} des_mesh_view;

/* Host copies of the Variables arrays the loop reads and writes
 * (parameters.hpp:270-280).  Any pointer not selected by a mask may be NULL. */
typedef struct des_state_view {
    int nnode, nelem;
    double *coord, *vel, *force, *coord0;             /* [nnode][3] */
    double *temperature, *mass, *tmass, *volume_n;    /* [nnode] */
    double *ntmp;                                     /* [nnode] */
    double *volume, *volume_old, *edvoldt;            /* [nelem] */
    double *plstrain, *delta_plstrain, *dpressure;    /* [nelem] */
    double *tmp_result_sg;                            /* [nelem] */
    double *stress, *strain, *strain_rate;            /* [nelem][6] */
    double *shpdx, *shpdy, *shpdz;                    /* [nelem][4] */
    double *tmp_result;                               /* [nelem][12] */
    double time, dt;
    int    steps;
} des_state_view;

/* Boundary topology in flat form; arrays are owned by the library. */
typedef struct des_topology {
    int       nnode, nelem;
    unsigned *bcflag;            /* [nnode]      create_boundary_flags (mesh.cxx:1529-1550) */
    int      *support_offsets;   /* [nnode+1]    create_support (mesh.cxx:1703-1717) as CSR */
    int      *support_elems;     /* [4*nelem]    ascending element id within a node */
    int      *support_slots;     /* [4*nelem]    local vertex index of the node in that element */
    int       bnodes_count[DES_NBDRY];
    int      *bnodes[DES_NBDRY];      /* create_boundary_nodes (mesh.cxx:1553-1573) */
    int       bfacets_count[DES_NBDRY];
    int      *bfacets[DES_NBDRY];     /* [count][2] (element, facet); create_boundary_facets (mesh.cxx:1633-1700) */
} des_topology;

typedef struct des_step_report {
    int       steps;
    double    time;
    double    dt;
    unsigned  status;            /* DES_STATUS_* bits accumulated since create/upload */
    long long ql_fallbacks;      /* elements that took the QL branch of dsyevh3 */
    long long eigen_solves;      /* elements whose principal stresses were computed */
    long long closure_candidates;   /* FP32 form with a closure: elements sent to the network */
    long long closure_accepted;     /* ... whose prediction passed the checks */
    long long exact_returns;        /* ... elements that took the exact FP64 return map */
} des_step_report;

typedef struct des_gpu des_gpu;

/* ---- host-only set-up (no GPU needed) ---------------------------------- */

/* Builds bcflag, support lists, bnodes and bfacets from connectivity, segment
 * and segflag, with the reference's ordering.  Replaces create_boundary_flags
 * (mesh.cxx:1542), create_boundary_nodes (mesh.cxx:1553),
 * create_boundary_facets (mesh.cxx:1633) and create_support (mesh.cxx:1703);
 * the facet search is a hash lookup instead of the O(nseg*nelem) scan. */
int  des_topology_build(const des_mesh_view *mesh, des_topology **out);
void des_topology_free(des_topology *topo);

/* Outward unit normals of the boundaries and the edge vectors of boundary
 * pairs, written into params->bnormals / params->edge_vectors.  Replaces
 * create_boundary_normals (bc.cxx:90-179); returns DES_ERR_OPTION where the
 * reference exits because a slanted (n0..n3) boundary is curved. */
int  des_boundary_normals(const des_topology *topo, const int *connectivity,
                          const double *coord, des_params *params);

/* ---- device handle ---------------------------------------------------- */

/* Allocates the device state for one mesh (replaces allocate_variables,
 * fields.cxx:13-54), uploads connectivity, boundary flags and material
 * tables and builds the support lists on the device (create_support,
 * mesh.cxx:1703-1717; the same lists as des_topology_build's).  device < 0
 * keeps the current device. */
int  des_gpu_create(const des_mesh_view *mesh, const des_params *params, int device,
                    des_gpu **out);
int  des_gpu_destroy(des_gpu *g);
int  des_gpu_set_params(des_gpu *g, const des_params *params);

/* The device's support lists (create_support, mesh.cxx:1703-1717), which
 * des_gpu_create and des_gpu_remesh build on the device from the
 * connectivity, copied into host arrays in des_topology's layout:
 * offsets[nnode+1], elems[4*nelem], slots[4*nelem].  Synchronises. */
int  des_gpu_download_support(des_gpu *g, int *offsets, int *elems, int *slots);

/* New per-element marker counts [nelem][nmat] (mesh->elemmarkers layout) for
 * the same mesh: the device's material tables follow the counts that
 * phase_changes (phasechanges.cxx:232-258) or a marker remap leaves in
 * var.elemmarkers, which MatProps reads through a reference
 * (matprops.cxx:165).  The reference calls compute_dt right after
 * phase_changes (dynearthsol.cxx:382-393): call des_gpu_compute_dt after this
 * at steps % 10 == 0.  Nodal masses stay those of the last update_mesh, as in
 * the reference; conductivities, densities and moduli of the next step follow
 * the new counts.  DES_ERR_TOPOLOGY for an element without markers (or a
 * negative count), DES_ERR_SIZE above 256 distinct count vectors,
 * DES_ERR_UNSUPPORTED when a closure is set and the counts change; the device
 * is unchanged after any error. */
int  des_gpu_set_elemmarkers(des_gpu *g, const int *elemmarkers);

/* The device half of remesh (remeshing.cxx:1963-2067).  The host has built the
 * new mesh, interpolated the fields and remapped the markers (new_mesh,
 * nearest_neighbor_interpolation, barycentric_node_interpolation,
 * remap_markers); mesh is the new mesh (connectivity, segments, segflag and
 * the remapped elemmarkers), host holds its interpolated fields: coord,
 * coord0, vel, temperature, plstrain, delta_plstrain, strain and stress.
 * The handle then holds a device state for the new mesh (support lists,
 * boundary flags and material tables rebuilt, reallocated fields zero as
 * reallocate_variables leaves them) and runs what remesh does after
 * reallocate_variables: compute_volume, volume_old = volume, compute_mass,
 * compute_shape_fn, and with reset_bottom_coord0 (remeshing_option 1, 2 or
 * 11) coord0 z = -zlength on the bottom boundary.  time, dt and steps, the
 * parameters (boundary normals included), the closure and the averaging
 * interval carry over.  For output during remeshing call
 * des_gpu_update_strain_rate and des_gpu_update_force after it, as remesh
 * does.  DES_ERR_UNSUPPORTED when a closure is set and the new mesh's marker
 * counts differ from the old; after any error the handle is unchanged. */
int  des_gpu_remesh(des_gpu *g, const des_mesh_view *mesh, const des_state_view *host,
                    int reset_bottom_coord0);

/* Host Variables -> device (fields in mask).  Marks nodal masses as current,
 * so the next step uses them as the reference does after update_mesh. */
int  des_gpu_upload(des_gpu *g, const des_state_view *host, unsigned mask);
/* device -> host Variables (fields in mask); synchronises. */
int  des_gpu_download(des_gpu *g, des_state_view *host, unsigned mask);

/* The init() sequence on the device after the mesh is in place
 * (dynearthsol.cxx:86-105): coord0 = coord, compute_volume, volume_old = volume,
 * compute_mass with T = 0, compute_shape_fn, apply_vbcs on zero velocity, then
 * the lithostatic initial_stress_state (ic.cxx:96-132).  Temperature and
 * plastic strain are taken from the last upload. */
int  des_gpu_init_fields(des_gpu *g);

/* Runs nsteps of the loop body dynearthsol.cxx:358-394 (without output,
 * remeshing, phase changes and hydration, which are no-ops for the supported
 * options) as one CUDA graph per step.  report may be NULL. */
int  des_gpu_step(des_gpu *g, int nsteps, des_step_report *report);

/* Drop-in form with host buffers: uploads the `mask` fields of host that the
 * loop body reads, runs nsteps, downloads all `mask` fields back.  The host
 * arrays stay authoritative, as in the reference loop.  Fields the loop body
 * overwrites before reading them (force, ntmp, strain_rate, dpressure,
 * edvoldt, tmp_result) are not uploaded; when coordinates, temperature,
 * volume, shape derivatives and masses are all in mask, the last three are
 * recomputed on the device from the uploaded coordinates and temperature
 * (update_mesh's own arithmetic, so the values equal what the previous step
 * left) and only volume_old is copied.  Page-locked host arrays
 * (des_host_register) are read in place by the upload.  The fields the last
 * step has finished before its last pass (coordinates, velocity, force,
 * temperature, plastic strain, strain rate, dpressure, edvoldt, ntmp) are
 * downloaded while that pass runs, so with DES_ERR_DT they may already hold
 * the step's values. */
int  des_gpu_step_host(des_gpu *g, des_state_view *host, unsigned mask, int nsteps,
                       des_step_report *report);

int  des_gpu_report(des_gpu *g, des_step_report *report);

/* ---- per-function entry points (resident state, reference semantics) -- */
int  des_gpu_update_temperature(des_gpu *g);   /* fields.cxx:108-172 */
int  des_gpu_update_strain_rate(des_gpu *g);   /* fields.cxx:175-247 */
int  des_gpu_compute_dvoldt(des_gpu *g);       /* geometry.cxx:117-151 (into ntmp) */
int  des_gpu_compute_edvoldt(des_gpu *g);      /* geometry.cxx:154-182 (from ntmp) */
int  des_gpu_update_stress(des_gpu *g);        /* rheology.cxx:513-654 */
int  des_gpu_NMD_stress(des_gpu *g);           /* geometry.cxx:185-254 */
int  des_gpu_update_force(des_gpu *g);         /* fields.cxx:312-375 + bc.cxx:503-595 + fields.cxx:250-309 */
int  des_gpu_update_velocity(des_gpu *g);      /* fields.cxx:378-393 */
int  des_gpu_apply_vbcs(des_gpu *g);           /* bc.cxx:182-500 */
int  des_gpu_update_coordinate(des_gpu *g);    /* fields.cxx:396-412 */
int  des_gpu_compute_volume(des_gpu *g);       /* geometry.cxx:86-114 */
int  des_gpu_compute_mass(des_gpu *g);         /* geometry.cxx:333-385 */
int  des_gpu_compute_shape_fn(des_gpu *g);     /* geometry.cxx:388-470 */
int  des_gpu_update_mesh(des_gpu *g);          /* dynearthsol.cxx:237-261 */
int  des_gpu_rotate_stress(des_gpu *g);        /* fields.cxx:455-533 */
int  des_gpu_compute_dt(des_gpu *g, double *dt_out);   /* geometry.cxx:257-330; also stores dt */

/* compute_volume (geometry.cxx:86-114) of any mesh given as host arrays in the
 * reference layout (coord [nnode][3], connectivity [nelem][4]) into host
 * volume[nelem], without a handle: the reference also calls it on meshes and
 * volume arrays that are not the loop's (markerset.cxx:238, remeshing.cxx:1069).
 * Copies the arrays to temporary device buffers, computes, copies back
 * (synchronous). */
int  des_compute_volume(int nnode, int nelem, const double *coord, const int *connectivity,
                        double *volume);

/* ---- learned return-map closure (no reference counterpart) -------------- */
/* A 14 -> 64 -> 64 -> 7 MLP with ReLU (inputs padded to 16, outputs to 8),
 * BF16 weights and activations with FP32 accumulation on the tensor cores.
 * It stands in for the Mohr-Coulomb shear return (rheology.cxx:180-240) of
 * the FP32 form.  Inputs (8 used), functions of the element's old stress,
 * strain increment and plastic strain: the principal values of the unit
 * deviator n of the elastic trial and the plastic strain capped at the
 * largest pls1, x = (raw - in_mean) * in_scale, each as a BF16 pair
 * (hi, 256 lo) (the temperature does not enter the shear return).  Outputs (4 used):
 * a, b D, c D and depls / |alam| with raw = y * out_scale, where the return
 * per unit plastic multiplier is (trial - new stress) / (2 G alam) =
 * a I + b n + c dev(n n) and D = (3 l_min^2 - 1)(3 l_max^2 - 1) clears the
 * poles of b and c; alam comes from the FP32 principal values of the
 * trial.  Weights are [out][in].  The des_mlp_* calls below take x and y
 * already normalised. */
#define DES_MLP_IN  16
#define DES_MLP_HID 64
#define DES_MLP_OUT 8
typedef struct des_mlp {
    float w1[DES_MLP_HID][DES_MLP_IN], b1[DES_MLP_HID];
    float w2[DES_MLP_HID][DES_MLP_HID], b2[DES_MLP_HID];
    float w3[DES_MLP_OUT][DES_MLP_HID], b3[DES_MLP_OUT];
    float in_mean[DES_MLP_IN], in_scale[DES_MLP_IN];
    float out_scale[DES_MLP_OUT];
    float env_lo[DES_MLP_IN], env_hi[DES_MLP_IN];   /* training envelope of x */
    float tol;                                      /* relative yield-residual tolerance */
} des_mlp;

/* y[n][8] = net(x[n][16]) on the tensor cores (host arrays). */
int  des_mlp_forward(const des_mlp *net, const float *x, long long n, float *y);
/* loss = mean over the n samples of the summed squared error of the 7
 * outputs, and its gradient with respect to every weight and bias. */
int  des_mlp_loss_grad(const des_mlp *net, const float *x, const float *y, long long n,
                       double *loss, des_mlp *grad);
/* Adam on the GPU for `steps` mini-batches of `batch` samples (shuffled once
 * with `seed`), the step size decaying along a cosine from lr to lr / 100;
 * net holds the initial and, on return, the trained weights.
 * loss_trace[steps] (may be NULL) receives the mini-batch losses. */
int  des_mlp_train(des_mlp *net, const float *x, const float *y, long long n, int steps,
                   int batch, float lr, unsigned long long seed, float *loss_trace);

/* ---- output frames ------------------------------------------------------ */
/* The state of Output::average_fields (output.cxx:227-267) over the current
 * averaging interval, AoS host arrays. */
typedef struct des_save_averages {
    const double *coord0;       /* [nnode][3] coordinates at the interval's first step */
    const double *strain0;      /* [nelem][6] strain at the interval's first step */
    const double *stress_sum;   /* [nelem][6] stress summed over the interval */
    const double *dpls_sum;     /* [nelem]    plastic-strain increments summed */
    double time0;               /* time at the interval's first step */
    int    interval;            /* mesh.quality_check_step_interval */
} des_save_averages;

/* One marker set (MarkerSet, markerset.hpp) as the output files hold it:
 * its name ("markerset" for the material markers), the number of markers,
 * the next id it would give out, and per marker the barycentric coordinates
 * in its element, the element, the material type and the id. */
typedef struct des_marker_set {
    const char   *name;
    int           nmarkers;
    int           last_id;
    const double *eta;          /* [nmarkers][4] */
    const int    *elem;         /* [nmarkers] */
    const int    *mattype;      /* [nmarkers] */
    const int    *id;           /* [nmarkers] */
} des_marker_set;

/* Writes the .save file of one output frame to `path` as Output::_write
 * (output.cxx:73-198, BinaryOutput binaryio.cxx:44-131) does, byte for byte:
 * avg NULL for Output::write_exact or when averaging is off; the nsets
 * marker sets last (MarkerSet::write_save_file, markerset.cxx:452-483: size,
 * marker coordinates from the nodes' coordinates, element, material, id) as
 * with sim.has_marker_output on (nsets = 0 for off).  Density, mesh quality,
 * viscosity, material and marker coordinates are computed on the host with
 * the reference's arithmetic.  Host-only; needs no GPU. */
int  des_write_save(const char *path, const des_mesh_view *mesh, const des_params *p,
                    const unsigned *bcflag, const des_state_view *s, const des_save_averages *avg,
                    const des_marker_set *sets, int nsets);

/* Asynchronous output (the download of output.cxx's fields overlapped with
 * the next steps): des_gpu_output_snapshot copies the `mask` fields
 * (DES_F_COORD, _VEL, _FORCE, _TEMPERATURE, _VOLUME, _STRESS, _STRAIN,
 * _STRAIN_RATE, _PLSTRAIN, _COORD0) as FP64 rows into device memory on the
 * step stream; des_gpu_output_fetch starts their copy to the host arrays of
 * `host` on a second stream and returns; steps may run meanwhile;
 * des_gpu_output_wait blocks until the copy is done and sets host's time, dt
 * and steps to the snapshot's.  The copies overlap only into page-locked
 * host memory (des_host_register). */
int  des_gpu_output_snapshot(des_gpu *g, unsigned mask);
int  des_gpu_output_fetch(des_gpu *g, des_state_view *host);
int  des_gpu_output_wait(des_gpu *g, des_state_view *host);

/* Writes the .chkpt file of a frame as Output::write_checkpoint
 * (output.cxx:270-296) does for a 3D model, its nsets marker sets last
 * (MarkerSet::write_chkpt_file, markerset.cxx:407-419: size and last id,
 * barycentric coordinates, element, material, id).  Host-only. */
int  des_write_checkpoint(const char *path, const des_mesh_view *mesh, double time,
                          double compensation_pressure, const double *volume_old,
                          const des_marker_set *sets, int nsets);

/* Output::average_fields on the device after every step from the next
 * des_gpu_step on (interval = mesh.quality_check_step_interval; 0 stops it). */
int  des_gpu_set_averaging(des_gpu *g, int interval);
/* The averaging state into host AoS arrays (any may be NULL) and *time0. */
int  des_gpu_download_averages(des_gpu *g, double *coord0, double *strain0, double *stress_sum,
                               double *dpls_sum, double *time0);

/* ---- remesh trigger: bad_mesh_quality on the device ------------------- */
typedef struct des_remesh_check {
    double smallest_size;            /* mesh.smallest_size */
    double resolution;               /* mesh.resolution */
    double zlength;                  /* mesh.zlength (the bottom is at -zlength) */
    double max_boundary_distortion;  /* mesh.max_boundary_distortion */
    double min_quality;              /* mesh.min_quality */
    int    remeshing_option;         /* mesh.remeshing_option */
} des_remesh_check;

/* bad_mesh_quality (remeshing.cxx:1893-1960) on the device state, with the
 * reference's order of checks: *code = 3 and *index = the first element
 * smaller than smallest_size * 0.118 * resolution^3; else 2 and the first
 * bottom node farther than max_boundary_distortion * resolution from the
 * bottom (remeshing options 1, 2, 11 only); else 1 and the first worst
 * element when the cube root of the worst elem_quality is below min_quality;
 * else 0.  *worst_quality (may be NULL) receives that cube root. */
int  des_gpu_bad_mesh_quality(des_gpu *g, const des_remesh_check *check, int *code, int *index,
                              double *worst_quality);
/* elem_quality (geometry.cxx:472-509) of every element into host
 * quality[nelem] (the "mesh quality" field of output.cxx:150-152). */
int  des_gpu_elem_quality(des_gpu *g, double *quality);

/* Records the inputs and outputs of every shear return the FP64 form makes
 * during nsteps steps (the training data of the closure; no reference
 * counterpart).  Each record is 24 floats: stress before [6], strain
 * increment [6], element temperature, plastic strain before, stress after
 * [6], plastic-strain increment, element index and step (int bits), the
 * dilation factor anpsi.  Up to `capacity` records are copied to `records`;
 * *count receives how many there were.  FP64 form only. */
int  des_gpu_log_returns(des_gpu *g, int nsteps, float *records, long long capacity,
                         long long *count);

/* Installs (net != NULL) or removes the learned closure in the FP32 form's
 * stress pass: network candidates are judged by their yield residual at
 * net->tol and fall back to the FP64 return map in the same kernel.  Needs
 * the FP32 form, rh_ep or rh_evp and one material mix (DES_ERR_UNSUPPORTED
 * otherwise).  The counts of candidates, accepted predictions and exact
 * returns accumulate in des_step_report. */
int  des_gpu_set_closure(des_gpu *g, const des_mlp *net);

/* ---- stable dt without any device allocation ---------------------------- */
/* Inputs of des_compute_dt_noalloc (the Param / MatProps values compute_dt
 * reads, geometry.cxx:257-330). */
typedef struct des_dt_inputs {
    double visc_min, therm_diff_max, max_vbc_val, inertial_scaling, dt_fraction, fixed_dt;
    double shear_modulus;   /* every element's shear modulus when shearm is NULL */
    double bulkm0, rho0;    /* bulkm(0) and rho(0); read only when not quasi-static */
    int    is_quasi_static, has_thermal_diffusion;
} des_dt_inputs;

/* No counterpart in the reference: an entry point for callers that cannot
 * call cudaMalloc (they manage all device memory themselves, or must not let
 * a library call cudaMalloc/cudaFree, which can synchronise the device).  It
 * computes the same dt as compute_dt from device arrays the caller passes in
 * the reference layout -- coord [nnode][3], connectivity [nelem][4] (16-byte
 * aligned), volume [nelem], optional per-element shear modulus -- and writes
 * it to the device double *dt, on `stream` (NULL: default stream), without
 * allocating anything.  `status` (a device int, may be NULL) receives DES_OK,
 * or DES_ERR_DT where compute_dt would exit with code 11 (dt <= 0,
 * geometry.cxx:321-325); read it after the stream has run the call.  Its
 * scratch is a fixed array inside the library: nelem is limited to
 * 16,777,216 (DES_ERR_SIZE above), calls that overlap on the GPU race, and
 * the first call on a device sets up the array's address (make it before any
 * stream capture; calls made outside a capture look the address up again, so
 * a device reset needs nothing more than one such call). */
int  des_compute_dt_noalloc(int nelem, const double *coord, const int *connectivity,
                            const double *volume, const double *shearm,
                            const des_dt_inputs *in, double *dt, int *status, void *stream);

/* ---- measurement (no reference counterpart) ----------------------------- */
/* Runs nsteps graph launches between two CUDA events on the handle's stream
 * and returns the elapsed device milliseconds (synchronises). */
int  des_gpu_time_steps(des_gpu *g, int nsteps, double *ms);
/* Runs nsteps with the six fused passes launched one by one, an event between
 * each, and returns the summed milliseconds of every pass in ms[6] (order
 * N-A, E-B, N-B, E-C, N-C, E-A).  Same results as des_gpu_step. */
int  des_gpu_profile_steps(des_gpu *g, int nsteps, double ms[6]);
/* Page-locks (or releases) caller memory so uploads and downloads run as
 * asynchronous DMA. */
int  des_host_register(void *ptr, long long bytes);
int  des_host_unregister(void *ptr);
/* sizeof of the ABI structs, for binding checks: params, mesh view, state
 * view, topology, step report */
void des_abi_sizes(long long out[5]);

/* ---- misc ------------------------------------------------------------- */
const char *des_gpu_error_string(int code);
/* bytes of device memory held by the handle */
long long   des_gpu_device_bytes(const des_gpu *g);
/* number of kernels one des_gpu_step launches per step */
int         des_gpu_kernels_per_step(const des_gpu *g);
/* Self-check of the integer-pipe FP64 arithmetic that the step kernels use
 * in place of FP64 unit instructions (no reference counterpart): n seeded
 * pseudo-random operands per kind on `device`, compared bit for bit with the
 * device's own FP64 instructions.  mismatches[0..9]: multiply on any bit
 * patterns, multiply on operands near 1, conversion to FP32 on any bit
 * patterns, conversion within the FP32 range, 0 + x, 2 x, x / 2, x / 6,
 * x / 3, x / 4 (the last six on any bit patterns and on exponents 0-8). */
int         des_gpu_softf64_check(int device, long long n, unsigned long long seed,
                                  unsigned long long mismatches[10]);

#ifdef __cplusplus
}
#endif
#endif /* DES_GPU_H */
