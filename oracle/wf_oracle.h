/*
 * wf_oracle.h — CPU oracle for the explicit SPH solid-mechanics step.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C FP64 restatement of
 * WeldFormGPU's kernel maths (src/cuda/InteractionAlt.cu, Mechanical.cu,
 * Functions.cu, tensor3.cu, Material.cuh, Thermal.cu, Contact.cu,
 * Geometry.cu, Mesh.cu; loop order from SolverFraser.cu) and of cuNSearch's
 * float32 neighbour rule (src/cuNSearch/src/cuNSearchKernels.cu).  Only the
 * tests, the smoke check and bench.py's CPU-baseline arm may load it; the
 * product library never does.
 *
 * Parity is pinned against the reference's own kernel sources compiled for
 * the CPU (oracle/_ref, built by oracle/build_ref.py) and against golden
 * vectors under tests/golden/ produced from them.
 *
 * The entry points mirror the product ABI (include/weldform_gb300.h) with a
 * `wfo_` prefix so that one scenario can be driven through both.
 */
#ifndef WF_ORACLE_H
#define WF_ORACLE_H

#include <stdint.h>
#include "../include/weldform_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct wfo_domain wfo_domain;

int         wfo_create(wfo_domain** out, int64_t particle_count);
int         wfo_destroy(wfo_domain* d);
const char* wfo_last_error(const wfo_domain* d);

int wfo_set_h(wfo_domain* d, double h);
int wfo_set_density(wfo_domain* d, double rho);
int wfo_set_shear_modulus(wfo_domain* d, double G);
int wfo_set_sigma_y(wfo_domain* d, double sy);
int wfo_set_conductivity(wfo_domain* d, double k);
int wfo_set_heat_cap(wfo_domain* d, double cp);
int wfo_set_cs(wfo_domain* d, const double* cs);
int wfo_set_free(wfo_domain* d, const uint8_t* is_free);
int wfo_set_id(wfo_domain* d, const int32_t* id);
int wfo_set_positions(wfo_domain* d, const double* x);
int wfo_set_velocities(wfo_domain* d, const double* v);
int wfo_set_mass(wfo_domain* d, const double* m);
int wfo_set_not_write_surf_id(wfo_domain* d, const uint8_t* flags);
int wfo_set_solid_count(wfo_domain* d, int64_t n_solid);
int wfo_set_time_step(wfo_domain* d, double dt);
int wfo_set_artificial_viscosity(wfo_domain* d, double alpha, double beta);
int wfo_set_material(wfo_domain* d, const wf_material* mat);
int wfo_add_velocity_bc(wfo_domain* d, int32_t zone_id, double vx, double vy, double vz);
int wfo_set_velocity_bc(wfo_domain* d, int32_t index, double vx, double vy, double vz);
/* output rows (same layout as wf_get_output_series), FP64 sums in index order */
int wfo_get_output_series(wfo_domain* d, double* rows, int64_t cap_rows, int64_t* n_rows,
                          int64_t* width);
int wfo_set_temperature(wfo_domain* d, const double* T);
int wfo_set_thermal_bc(wfo_domain* d, const int32_t* bc_t);
int wfo_set_convection(wfo_domain* d, double h_conv, double T_inf);
int wfo_set_option(wfo_domain* d, const char* key, double value);
/* contact with rigid triangle meshes (src/cuda/Contact.cu, Geometry.cu, Mesh.cu) */
int wfo_set_contact(wfo_domain* d, double mu_static, double mu_dynamic, int law);
int wfo_add_trimesh(wfo_domain* d, const double* nodes, int32_t nn, const int32_t* tris,
                    int32_t ne, const double* normals, int32_t zone_id, int64_t first,
                    const double* vel, const double* angvel);
int64_t wfo_gen_plane_mesh(int axis, int positive, const double* p1, const double* p2, int dens,
                           double* nodes, int32_t* tris, double* normals);
int wfo_set_threads(int nthreads);

int wfo_mech_fraser_solve(wfo_domain* d, double tf, double dt_out);
int wfo_thermal_solve(wfo_domain* d, double tf);
int wfo_step(wfo_domain* d, int64_t nsteps);
int wfo_find_neighbors(wfo_domain* d);
/* Runs one named stage of the Fraser loop body on the current state
 * ("density", "update_density", "rates", "pressure", "stress", "accel",
 * "bc", "update_pos", "update_vel", "thermal", "energy"). */
int wfo_run_stage(wfo_domain* d, const char* stage);
/* GradKernel (cubic spline, Dim 3): the scalar GK with grad W = GK * x_ij. */
double wfo_grad_kernel(double q, double h);

int wfo_get_field(wfo_domain* d, const char* name, double* out);
int wfo_get_field_i32(wfo_domain* d, const char* name, int32_t* out);
int wfo_get_neighbors(wfo_domain* d, int32_t* counts, int32_t* lists);
int wfo_get_scalar(wfo_domain* d, const char* name, double* out);
int wfo_set_field(wfo_domain* d, const char* name, const double* in);

/* ---- particle generators (host domain setup, src/Domain.cpp) ---------- */
/* Domain::AddCylinderLength (src/Domain.cpp:490-573).  Two-call protocol:
 * pass x == NULL to get the count.  Returns the count; *mass is the
 * per-particle mass the reference assigns. */
int64_t wfo_gen_cylinder_ref(double x0, double y0, double z0, double Rxy, double Lz,
                             double r, double density, double* x, double* mass);
/* Domain::AddBoxLength, cubic packing (type 1), src/Domain.cpp:194-398. */
int64_t wfo_gen_box_cubic(double x0, double y0, double z0, double Lx, double Ly, double Lz,
                          double r, double density, double* x, double* mass);
/* Cubic lattice of spacing dx inside a cylinder (axis z, base at z0), with
 * seeded uniform jitter of +-jitter*dx per coordinate (splitmix64). */
int64_t wfo_gen_cylinder_uniform(double Rxy, double Lz, double r, double density, double ang,
                                 int rows, double r_i, int32_t tag, double* x, int32_t* ids,
                                 double* mass);
int64_t wfo_gen_cylinder_lattice(double R, double H, double dx, double jitter,
                                 uint64_t seed, double* x);
/* Domain::AssignZone (src/Domain.cpp:989-1005): returns the count tagged. */
int64_t wfo_assign_zone(const double* x, int64_t n, const double* start, const double* end,
                        int32_t zone_id, int32_t* id, uint8_t* not_write);

/* ---- MLP warm start for the Johnson-Cook return map (FP64 reference) ---- */
/* Layer sizes 4 -> 64 -> 64 -> 1, SiLU hidden activations.  Parameters are
 * packed W1[64*4], b1[64], W2[64*64], b2[64], W3[64], b3[1] (row-major,
 * out x in).  Forward for `n` samples of 4 inputs. */
#define WFO_MLP_NPARAM (64 * 4 + 64 + 64 * 64 + 64 + 64 + 1)
int wfo_set_mlp_params(wfo_domain* d, const double* params);
int wfo_mlp_forward(const double* params, const double* xin, int64_t n, double* yout);
/* Mean-squared-error loss over a batch and its gradient wrt every parameter. */
int wfo_mlp_loss_grad(const double* params, const double* xin, const double* target,
                      int64_t n, double* loss, double* grad);

#ifdef __cplusplus
}
#endif
#endif
