/*
 * weldform_gb300.h — C ABI of the GB300-native explicit SPH solid-mechanics step.
 *
 * The library replaces the device half of WeldFormGPU's `SPH::Domain_d`
 * (src/cuda/Domain_d.cuh:101-426): the same setters, the same solve entry
 * points (MechFraserSolve / MechSolve / ThermalSolve) and the same physics,
 * behind plain C functions that take host pointers and sizes.  Every entry
 * point names the reference member or host statement it replaces.
 *
 * Conventions
 *   - Every function returns an int status: WF_OK (0) or a negative WF_ERR_*.
 *     No function exits the process; wf_last_error() describes the failure.
 *   - Arrays of per-particle vectors are interleaved xyz (like double3[n]);
 *     symmetric tensors are 6 values per particle in the reference's flat
 *     order [xx, yy, zz, xy, yz, xz] (src/cuda/tensor3.cu:95-100).
 *   - Host pointers are only read (or written, for getters) during the call.
 *   - Particle indices at the ABI are the caller's original indices; the
 *     library keeps its own cell-sorted order on the device.
 *   - One handle per host thread; a handle owns one CUDA stream.
 */
#ifndef WELDFORM_GB300_H
#define WELDFORM_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define WF_OK            0
#define WF_ERR_ARG      -1   /* bad argument (null pointer, size, unknown name)      */
#define WF_ERR_CUDA     -2   /* CUDA runtime error                                   */
#define WF_ERR_STATE    -3   /* call made in the wrong state (e.g. no positions)     */
#define WF_ERR_ALLOC    -4   /* device or host allocation failed                     */
#define WF_ERR_NUMERIC  -5   /* a kernel reported NaN/Inf or an overflowed list       */
#define WF_ERR_IO       -6   /* file could not be opened / parsed                    */

/* Neighbour-list capacity per particle: CUDA_MAX_NEIGHBORS
 * (src/cuNSearch/src/cuNSearchKernels.cuh:6). */
#define WF_MAX_NEIGHBORS 70

/* Material model ids: src/cuda/Material.cuh:6-8. */
#define WF_BILINEAR      0
#define WF_HOLLOMON      1
#define WF_JOHNSON_COOK  2

/* Material constants, in the JSON `const[]` order the reference reads
 * (src/WeldFormGPU.cu:753-792): bilinear const[0] = Et; JC const[] =
 * [A, B, n, C, eps_0, m, T_m, T_t]; Hollomon const[] = [K, m]. */
typedef struct wf_material {
  int32_t model;
  int32_t reserved;
  double  E;        /* youngsModulus                                  */
  double  nu;       /* poissonsRatio                                  */
  double  sy0;      /* yieldStress0 (initial sigma_y, Hollomon sy0)   */
  double  Et;       /* bilinear tangent modulus                       */
  double  K_hol;    /* Hollomon K                                     */
  double  m_hol;    /* Hollomon exponent m                            */
  double  A, B, n, C, eps0, m, Tm, Tt;   /* Johnson-Cook             */
} wf_material;

typedef struct wf_domain wf_domain;

/* ---- lifecycle ------------------------------------------------------- */
/* Domain_d::SetDimension (src/cuda/Domain_d.cu:19-234): allocates the SoA
 * arena for `particle_count` particles; solid_part_count = particle_count. */
int         wf_create(wf_domain** out, int64_t particle_count);
/* Domain_d::~Domain_d.  The domain's device arena (one allocation for every
 * per-particle array) is kept for the next wf_create on the same device whose
 * layout needs between 80 and 100 % of it (zeroed there like a fresh one);
 * wf_release_cache() returns it to the driver. */
int         wf_destroy(wf_domain* d);
int         wf_release_cache(void);
const char* wf_last_error(const wf_domain* d);
const char* wf_version(void);

/* ---- reference setters (src/cuda/Domain_d.cu:307-477) ----------------- */
int wf_set_h(wf_domain* d, double h);                /* Set_h        :416 */
int wf_set_density(wf_domain* d, double rho);        /* SetDensity   :458 (rho and rho_0) */
int wf_set_shear_modulus(wf_domain* d, double G);    /* SetShearModulus :447 */
int wf_set_sigma_y(wf_domain* d, double sy);         /* SetSigmay    :437 */
int wf_set_conductivity(wf_domain* d, double k);     /* SetConductivity :427 */
int wf_set_heat_cap(wf_domain* d, double cp);        /* SetHeatCap   :469 */
int wf_set_cs(wf_domain* d, const double* cs);       /* SetCs        :331 (per particle) */
int wf_set_free(wf_domain* d, const uint8_t* is_free);   /* SetFreePart :307 */
int wf_set_id(wf_domain* d, const int32_t* id);          /* SetID       :317 */

/* ---- public fields the reference's main writes directly --------------- */
/* rejects non-finite positions (WF_ERR_ARG, nothing written); after a solve
 * has started, the next step rebuilds the lists for the new positions */
int wf_set_positions(wf_domain* d, const double* x);     /* cudaMemcpy x, WeldFormGPU.cu:704 */
int wf_set_velocities(wf_domain* d, const double* v);    /* cudaMemcpy v, WeldFormGPU.cu:711 */
int wf_set_mass(wf_domain* d, const double* m);          /* cudaMemcpy m, WeldFormGPU.cu:822 */
int wf_set_not_write_surf_id(wf_domain* d, const uint8_t* flags); /* WeldFormGPU.cu:858 */
int wf_set_solid_count(wf_domain* d, int64_t n_solid);   /* solid_part_count, WeldFormGPU.cu:453 */
int wf_set_time_step(wf_domain* d, double dt);           /* deltat, WeldFormGPU.cu:906 */
int wf_set_artificial_viscosity(wf_domain* d, double alpha, double beta); /* Alpha/Beta :292 */
int wf_set_material(wf_domain* d, const wf_material* mat);    /* materials[0], WeldFormGPU.cu:749-800 */
int wf_add_velocity_bc(wf_domain* d, int32_t zone_id,
                       double vx, double vy, double vz);  /* bConds, WeldFormGPU.cu:457-485 */
/* Changes the velocity of BC number `index` (0-based, in wf_add_velocity_bc
 * order), e.g. from a callback between steps: the reference's UserAcc
 * (src/WeldFormGPU.cu:78-140) writes bConds[bc].value each step. */
int wf_set_velocity_bc(wf_domain* d, int32_t index, double vx, double vy, double vz);
int wf_set_temperature(wf_domain* d, const double* T);   /* T (Domain_d::CopyData, Domain_d.cu:490) */
int wf_set_thermal_bc(wf_domain* d, const int32_t* bc_t); /* BC_T: 0 none, 1 convection */
int wf_set_convection(wf_domain* d, double h_conv, double T_inf); /* h_conv_double, T_inf */

/* ---- contact with rigid triangle meshes ---------------------------------
 * friction_sta / friction_dyn (src/WeldFormGPU.cu:631-641, Domain_d.cuh:260)
 * and the contact law: 0 = the reference's penalty law
 * (CalcContactForcesWang, src/cuda/Contact.cu:134-321); 1 = a law with no
 * reference counterpart, for tools of many triangles: each solid particle
 * takes its nearest triangle within h (triangles binned in cells that move
 * with the tool), the gap to the nearest surface point along the direction
 * from that point (the face normal for a centre behind the face), penalty
 * F_n = contact_stiffness * K * contact_dx * (contact_dx/2 - gap), Coulomb
 * friction -mu_static F_n v_t / max(|v_t|, contact_vreg) with v_t the
 * tangential velocity relative to the tool surface at the nearest point
 * (m_v + m_w x q), and frictional heat contact_heat_fraction * mu_static F_n
 * |v_t|^2 / max(|v_t|, contact_vreg) into the particle ("fric_heat", W).
 * Translating tools are binned once, rotating ones again on the GPU every
 * step.  Law 1 needs the option contact_dx (the solve fails with WF_ERR_STATE
 * without it) and meshes of fewer than 2^24 triangles. */
int wf_set_contact(wf_domain* d, double mu_static, double mu_dynamic, int law);
/* A rigid triangle mesh (TriMesh_d, src/cuda/Mesh.cuh:19-54) as main adds it
 * (AddTrimeshParticles + AssignTrimeshAddress + SetMeshVel,
 * src/WeldFormGPU.cu:545-610): particles first .. first+ne-1, which must
 * follow the solid ones (wf_set_solid_count), become the element centroids
 * with mass 0 and the mesh's zone id; the mesh moves with velocity `vel`
 * and angular velocity `angvel` (m_v, m_w).  nodes: 3*nn doubles; tris:
 * 3*ne node indices; normals: 3*ne doubles or NULL (computed as
 * TriMesh_d::CalcNormals).  Call after wf_set_positions and wf_set_mass;
 * turns contact on (surface tagging, contact list, penalty forces, mesh
 * motion in MechFraserSolve order).  Zone id 1 is the free-surface id. */
int wf_add_trimesh(wf_domain* d, const double* nodes, int32_t nn, const int32_t* tris,
                   int32_t ne, const double* normals, int32_t zone_id, int64_t first,
                   const double* vel, const double* angvel);

/* Options with no reference field; the defaults reproduce the reference and
 * unknown keys fail with WF_ERR_ARG.  Keys (default):
 *   precision (0 FP64, 1 mixed), return_map (0 radial, 1 Newton),
 *   newton_rtol (1e-10), newton_max_iter (50, >= 1; a return map that stops
 *   there unconverged is counted ("newton_capped") and the call returns
 *   WF_ERR_NUMERIC, the state advanced with the unconverged increments),
 *   mlp (0), log_return_map (0),
 *   output_every_step (0: output rows at output times only), print_outputs
 *   (0: 1 prints MechFraserSolve's lines at output times), output_series_cap
 *   (65536 rows),
 *   rebuild_every (5), rebuild_after_yield (1), rebuild_current_positions (0),
 *   rebuild_strain_increment (0), thermal (0), taylor_quinney (0),
 *   clamp_homologous (1), energy_mode (0: particle 0's S:D for every
 *   particle, as Energy.cu:270-276; 1: each particle's own; both forms),
 *   contact_dx (0),
 *   contact_stiffness (0.1), contact_vreg (1e-3), contact_heat_fraction (1),
 *   fuse_heat (1), fuse_integrate (1), tile_staging (0; 1: the mixed pair passes
 *   read neighbours from per-tile halos in shared memory; same results),
 *   tile_cap_max (2048: largest halo staged), list_prefetch (2: L2 prefetch of
 *   the neighbour lists that many blocks ahead; 0 off), state_prefetch (1: L2 prefetch, before
 *   the pair loop, of the state each mixed pass reads after it), wave_prefetch
 *   (2: L2 prefetch of the prologue and first 2 list blocks of the slot one
 *   resident wave of blocks later; 0 off), wave_prefetch_distance (1.0, in
 *   resident waves), list16 (0; 1: 16-bit list offsets for
 *   the mixed passes' global gathers; same results), graph (1), output_interval (1e300),
 *   resume (0), profile_kernel (0), debug_checks (0; 1: after every rebuild each
 *   neighbour list is checked before any pass reads it, a bad entry replaced by the
 *   particle's own slot, and after every step positions and velocities are checked
 *   for non-finite values; either sets status bit 6 and the call returns
 *   WF_ERR_STATE), debug_inject_list_error (a particle id: its list's first entry is
 *   set out of range after the next list build, for testing the checks; only with
 *   debug_checks = 1). */
int wf_set_option(wf_domain* d, const char* key, double value);

/* The per-step BC hook: Domain_d::GeneralAfter (src/cuda/Domain_d.cuh:402,
 * set to UserAcc at src/WeldFormGPU.cu:688).  `fn` runs on the calling host
 * thread after every step of a solve (wf_mech_fraser_solve, wf_step,
 * wf_time_steps), when the step's device work is ordered before any later
 * call on the handle; d->time is then the time of the next step.  It may call
 * the getters and setters of this handle (wf_get_field, wf_set_velocity_bc,
 * wf_set_field, ...) but not its solvers.  A non-zero return ends the solve
 * with WF_ERR_STATE.  While a callback is set the steps are launched one by
 * one (no step graphs).  fn = NULL removes it. */
typedef int (*wf_after_fn)(wf_domain* d, void* user);
int wf_set_callback(wf_domain* d, wf_after_fn fn, void* user);

/* ---- solvers ------------------------------------------------------------ */
/* Domain_d::MechFraserSolve (src/cuda/SolverFraser.cu:30-409). */
int wf_mech_fraser_solve(wf_domain* d, double tf, double dt_out);
/* Domain_d::MechSolve (declared at src/cuda/Domain_d.cuh:310, never
 * defined): bound to the Fraser loop. */
int wf_mech_solve(wf_domain* d, double tf, double dt_out);
/* Domain_d::ThermalSolve (src/cuda/Thermal.cu:188-260). */
int wf_thermal_solve(wf_domain* d, double tf);
/* `nsteps` iterations of the Fraser loop body (SolverFraser.cu:164-398). */
int wf_step(wf_domain* d, int64_t nsteps);
/* Rebuild the neighbour list now (cuNSearch find_neighbors, cuNSearch.cu:111). */
int wf_find_neighbors(wf_domain* d);

/* Neighbour search that allocates no device memory.  No counterpart in the
 * reference.  For callers that cannot call cudaMalloc: hosts whose framework
 * owns every device allocation (its own pool or allocator), hosts held to a
 * device-memory budget reserved up front, and code that must not allocate
 * while other work runs on the GPU.  Gives the lists of wf_find_neighbors +
 * wf_get_neighbors for the same positions and h: radius 2h, cuNSearch's
 * float32 rule, candidates in the z, y, x cell order, ascending index inside a
 * cell, at most WF_MAX_NEIGHBORS per particle (a count of 70 may mean the list
 * was cut, as in the reference).
 *   x       device, 3*n doubles, interleaved xyz (read only)
 *   counts  device, n int32 (written)
 *   lists   device, n*WF_MAX_NEIGHBORS int32, row-major; row i holds particle
 *           i's neighbour indices, entries past counts[i] are left untouched
 *   stream  cudaStream_t to run on (NULL: the legacy default stream); the call
 *           returns once the lists are written (it waits for the stream twice)
 *   err     optional buffer of err_len bytes for a one-line message
 * Temporaries live in one fixed device array inside the library,
 * WF_STATIC_SCRATCH_BYTES (about 4.5 MiB), which every GPU that loads the
 * library holds until the process exits.  Limits: n <= WF_STATIC_MAX_PARTICLES
 * and a search grid (bounding box in cells of size 2h, plus a margin of two
 * cells a side) of at most WF_STATIC_MAX_CELLS cells; larger inputs fail with
 * WF_ERR_ARG and a message naming the limit.  The first call on each device
 * looks up the array's device address (cudaGetSymbolAddress) for the device
 * current at the call and caches it: make that first call before any stream
 * capture.  All calls share the array and each call overwrites what the last
 * one left there: calls whose GPU work overlaps on one device (two streams or
 * two host threads at once) race and give wrong lists, so serialise them. */
#define WF_STATIC_MAX_PARTICLES 65536
#define WF_STATIC_MAX_CELLS     262144
#define WF_STATIC_SCRATCH_BYTES 4723200
int wf_find_neighbors_static(const double* x, int64_t n, double h, int32_t* counts,
                             int32_t* lists, void* stream, char* err, int64_t err_len);

/* ---- outputs (caller's particle order) --------------------------------- */
int wf_get_field(wf_domain* d, const char* name, double* out);
int wf_get_field_i32(wf_domain* d, const char* name, int32_t* out);
/* counts[n]; lists[n*WF_MAX_NEIGHBORS], neighbour ids in search order. */
int wf_get_neighbors(wf_domain* d, int32_t* counts, int32_t* lists);
/* "time", "step", "is_yielding", "isfirst", "launches", "rebuilds" (neighbour
 * rebuilds inside the step loop), "newton_iters", "newton_calls", "mlp_used",
 * "newton_capped" (return maps that stopped at newton_max_iter), "status",
 * "int_energy_sum", "contact_tests32" / "contact_tests64" (contact
 * law 1: triangle tests in the FP32 search and the FP64 decision, since
 * creation); from the last output row: "max_disp_x|y|z", "max_pl_strain",
 * "cont_force_sum", "cont_force_x|y|z", "int_energy_total",
 * "reaction_x|y|z" (BC 0). */
int wf_get_scalar(wf_domain* d, const char* name, double* out);

/* ---- output reductions ------------------------------------------------------
 * MechFraserSolve reduces the state on the host at every output time
 * (src/cuda/SolverFraser.cu:350-388: max displacement, max plastic strain,
 * the contact force sum over free-surface particles).  Here the same values
 * and the load each velocity BC carries are reduced on the device in FP64, in
 * an order fixed by the particle count alone (original ids, fixed blocks),
 * into one row per output time (every step with option output_every_step):
 *   [0] time, [1] step, [2..4] max u_x, u_y, u_z (from 0, as the reference),
 *   [5] max pl_strain, [6] sum of |contforce| over ID == 1 particles,
 *   [7..9] contact force vector sum, [10] internal energy sum,
 *   [11 + 3b .. 13 + 3b] BC b's reaction: the sum over its zone of m a
 *   before the BC zeroes a (the force the rest of the body puts on the zone;
 *   the platen supplies its negative).
 * Rows of a solve are kept in order (up to output_series_cap, later rows are
 * dropped and status bit 32 set); a solve that does not resume starts a new
 * series.  With CSV output on (wf_set_csv_output), MechFraserSolve writes
 * the series to <prefix>outputs.csv at its end. */
#define WF_ROW_FIXED_COLUMNS 11
/* the last row recorded (cap values at most); *width = row width.  WF_ERR_STATE
 * before the first row. */
int wf_get_output_row(wf_domain* d, double* row, int64_t cap, int64_t* width);
/* up to cap_rows rows of the series, row-major; *n_rows = rows copied (with
 * cap_rows = 0: rows stored) */
int wf_get_output_series(wf_domain* d, double* rows, int64_t cap_rows, int64_t* n_rows,
                         int64_t* width);
/* BC `bc_index`'s reaction (3 doubles) from the last row */
int wf_get_reaction(wf_domain* d, int32_t bc_index, double* force);
/* Checkpoint / restart (no reference counterpart: the reference's CSV
 * snapshots are not restartable).  wf_set_field writes a state field in the
 * caller's order (names as wf_get_field; "x" goes through wf_set_positions,
 * which rejects non-finite values, and after the first solve step makes the
 * next step rebuild the neighbour lists); wf_set_scalar sets "time",
 * "step", "isfirst" or "is_yielding"; with wf_set_option("resume", 1) the
 * next solve keeps time and velocities instead of restarting from rest. */
int wf_set_field(wf_domain* d, const char* name, const double* in);
int wf_set_scalar(wf_domain* d, const char* name, double value);
/* Domain_d::WriteCSV (src/cuda/Domain_d.cu:556-587), same columns. */
int wf_write_csv(wf_domain* d, const char* path);
/* MechFraserSolve's snapshots (SolverFraser.cu:142-144, 357-360): with a
 * non-NULL prefix, solves write <prefix>out_<time %.6f>.csv at their start
 * and at every output time; NULL turns them off (the default). */
int wf_set_csv_output(wf_domain* d, const char* prefix);

/* ---- the reference's input-file driver ---------------------------------
 * main of src/WeldFormGPU.cu:142-926: reads the reference's JSON keys
 * (Configuration, Materials, DomainBlocks Box / Cylinder, DomainZones,
 * DomainBlocks File (an LS-DYNA keyword deck, wf_read_lsdyna),
 * RigidBodies Plane / File (Nastran), Contact, BoundaryConditions), builds and sets up the
 * domain as main does, runs MechFraserSolve(simTime, outTime) writing
 * out_<time>.csv into out_dir and test.csv at the end.  err (optional,
 * err_len bytes) receives a one-line message on failure.  Keys with no
 * reference counterpart: Configuration.precision ("fp64" | "mixed"),
 * returnMap ("radial" | "newton"), solver "Mech-Thermal" with
 * Materials.thermalCond / thermalHeatCap and taylorQuinney,
 * InitialConditions[0].Temp. */
int wf_run_json(const char* path, const char* out_dir, char* err, int64_t err_len);

/* ---- host domain set-up (src/Domain.cpp) --------------------------------- */
/* Two-call protocol: pass x == NULL to get the particle count, then a buffer
 * of 3*count doubles.  Return value: the count. */
/* Domain::AddCylinderLength (src/Domain.cpp:490-573); *mass = pi R^2 Lz rho / N */
int64_t wf_gen_cylinder(double x0, double y0, double z0, double Rxy, double Lz, double r,
                        double density, double* x, double* mass);
/* Domain::AddBoxLength, cubic packing (src/Domain.cpp:296-338) */
int64_t wf_gen_box(double x0, double y0, double z0, double Lx, double Ly, double Lz, double r,
                   double density, double* x, double* mass);
/* Domain::AddCylUniformLength (src/Domain.cpp:1071-1192), the reference's
 * "Cylindrical" grid: rings of ceil(ang ri / 2r) particles at radii r_i,
 * r_i + 2r, ... < Rxy in rows z = r, 3r, ... (axis z, base z = 0); ids
 * `tag`, 2 / 3 on the first / last `rows` of a slice (ang < 2 pi), 4 on the
 * axis; *mass = pi Rxy^2 Lz density / count.  Two-call protocol. */
int64_t wf_gen_cylinder_uniform(double Rxy, double Lz, double r, double density, double ang,
                                int rows, double r_i, int32_t tag, double* x, int32_t* ids,
                                double* mass);
/* Cubic lattice of spacing dx clipped to a cylinder (axis z, base z = 0),
 * jittered by U[-jitter, jitter]*dx per coordinate from a splitmix64 stream;
 * no reference counterpart (synthetic benchmark workload). */
int64_t wf_gen_cylinder_lattice(double R, double H, double dx, double jitter, uint64_t seed,
                                double* x);
/* TriMesh_d::AxisPlaneMesh (src/cuda/Mesh.cu:48-194) as main builds a
 * "Plane" rigid body (src/WeldFormGPU.cu:545-552): (dens+1)^2 nodes stepped
 * by (p2[0] - p1[0])/dens in x and y from p1 at z = p1[2], 2 dens^2
 * triangles ordered for a normal along +axis when `positive` (main passes
 * axis 2, positive 0).  Returns the triangle count; nodes (3 (dens+1)^2),
 * tris (3 per triangle) and normals (3 per triangle) are written when not
 * NULL. */
int64_t wf_gen_plane_mesh(int axis, int positive, const double* p1, const double* p2, int dens,
                          double* nodes, int32_t* tris, double* normals);
/* Icosphere tool (no reference counterpart: the rigid indenter of the
 * 2M-particle contact workload): radius R about center[3], the icosahedron
 * split `level` times (20 * 4^level faces), outward normals; lower_half keeps
 * the faces at or below center[2].  Returns the face count and *n_nodes;
 * fills nodes / tris when not NULL. */
int64_t wf_gen_icosphere(double R, const double* center, int level, int lower_half,
                         double* nodes, int32_t* tris, int64_t* n_nodes);
/* NastranReader::read (src/NastranReader.cpp:5-150) + TriMesh_d::
 * ReadFromNastran (src/cuda/Mesh_reader.cu:5-100): fixed-field GRID / CTRIA
 * cards with implicit exponents ("0.7354-03").  Returns the triangle count
 * (negative WF_ERR_IO / WF_ERR_ARG on a missing file, beam elements or an
 * unknown node id) and *n_nodes; with nodes (3 n_nodes) and tris (3 per
 * triangle, node positions) not NULL, fills them. */
int64_t wf_read_nastran(const char* path, double* nodes, int32_t* tris, int64_t* n_nodes);
/* Domain_d::ReadFromLSdyna (src/cuda/Domain_d.cu:236-281; the reference reads
 * through the LSDynaReader submodule, absent from its tree, so this follows
 * the public LS-DYNA keyword format): one particle per *ELEMENT_SPH card (NID,
 * PID, MASS in fields of 8, 8, 16 characters, or comma-separated), in card
 * order, at the position of its *NODE card (NID, X, Y, Z in fields of 8, 16,
 * 16, 16, or comma-separated), with the card's mass; a particle whose node is
 * listed in a *SET_NODE_LIST[_TITLE] (SID on its first card, node ids in
 * fields of 10 on the following cards) takes the set's id, a later set
 * overriding an earlier one, others 0.  '$' lines are comments.  Two-call
 * protocol: with x, mass and ids NULL returns the particle count.  Negative:
 * WF_ERR_IO (missing file, unreadable card), WF_ERR_ARG (no SPH element, an
 * element naming an unknown node). */
int64_t wf_read_lsdyna(const char* path, double* x, double* mass, int32_t* ids);
/* Domain::AssignZone (src/Domain.cpp:989-1005): tags particles inside the
 * inclusive box [start, end]; returns how many. */
int64_t wf_assign_zone(const double* x, int64_t n, const double* start, const double* end,
                       int32_t zone_id, int32_t* id, uint8_t* not_write);

/* ---- learned warm start of the Johnson-Cook return map ------------------
 * No reference counterpart (the reference's return map is a one-shot radial
 * return, src/cuda/Mechanical.cu:503-536).  A 4 -> 64 -> 64 -> 1 SiLU MLP
 * proposes dlambda / dlambda_radial; Newton still converges to the same
 * tolerance.  Parameters: float[4545] = W1[64*4], b1[64], W2[64*64], b2[64],
 * W3[64], b3 (row-major, out x in); features: float4 per sample. */
#define WF_MLP_NPARAMS 4545
/* loads trained parameters into the domain; enable with option "mlp" = 1 */
int wf_set_mlp_weights(wf_domain* d, const float* params);
/* (features, dlambda/dlambda_radial) pairs logged by the plain FP64 solver
 * while option "log_return_map" (capacity) is set: copies up to cap pairs */
int wf_get_return_map_log(wf_domain* d, float* X, float* Y, int64_t cap, int64_t* count);
/* Y = network(X) for n samples: use_tensor_cores != 0 runs the tcgen05 path of
 * the solver (BF16 operands, FP32 accumulation), 0 an FP32 reference kernel. */
int wf_mlp_infer(const float* params, const float* X, int64_t n, int use_tensor_cores, float* Y);
/* mean-squared-error loss and its gradient over n samples (training kernels) */
int wf_mlp_grad(const float* params, const float* X, const float* Y, int64_t n, float* grad,
                float* loss);
/* Adam with cosine decay over `steps` mini-batches; params updated in place */
int wf_mlp_train(float* params, const float* X, const float* Y, int64_t n, int64_t steps,
                 int64_t batch, float lr, float* final_loss);
/* synthetic states (ratio U[1,3], eps_p log-U[1e-4,2], rate log-U[1e-2,1e5],
 * T U[20,550]) with their converged increments: features X, targets Y,
 * raw states (ratio, eps_p, rate, T) and the Newton iterations from the
 * radial start */
int wf_mlp_synth(const wf_material* mat, double G, int64_t n, uint64_t seed, double rtol,
                 float* X, float* Y, float* states, int32_t* iters_radial);
/* Newton iterations on given raw states from the network's start
 * (params != NULL, BF16 tensor cores) or the radial start; used[i] = 1 when
 * the network's prediction was taken; dl = converged increment */
int wf_mlp_newton_iters(const wf_material* mat, double G, const float* params,
                        const float* states, int64_t n, double rtol, int32_t* iters,
                        int32_t* used, float* dl);

/* ---- measurement -------------------------------------------------------- */
/* Runs `nsteps` steps on the handle's stream between CUDA events and
 * returns the elapsed device time; per-kernel event pairs are recorded
 * around the kernel named by wf_set_option("profile_kernel", id). */
int wf_time_steps(wf_domain* d, int64_t nsteps, double* elapsed_ms,
                  double* kernel_ms, int64_t* kernel_launches,
                  int64_t* total_launches);
/* Throughput of the FP64 fused multiply-add pipe of the current device in
 * GFLOP/s (2 flops per FMA), measured with CUDA events over independent FMA
 * chains on every SM: the arithmetic ceiling of the plain FP64 form (no
 * reference counterpart). */
int wf_fp64_fma_peak(double* gflops, double* ms_per_launch);

#ifdef __cplusplus
}
#endif

#endif /* WELDFORM_GB300_H */
