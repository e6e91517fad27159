/*
 * vsim_oracle.h -- TEST INFRASTRUCTURE ONLY.
 *
 * A CPU restatement of the visionary-sim reference's solver step (its WGSL
 * compute shaders and the JS that feeds them), the oracle the GPU library's
 * results are compared against and the timed CPU baseline. Nothing in the product links,
 * loads or calls this; only tests/, __graft_entry__.smoke() and bench.py's
 * CPU legs do.
 *
 * Parity pins: the reference has no runnable CPU step (its unit-test compute
 * backend is a no-op, packages/visionary-sim/test/helpers/fakeCompute.js:5-31)
 * and no Node runtime exists here, so the oracle is pinned by porting the
 * reference's own known-answer tests (elastic, contact, kinematicDrive,
 * stretch, sample, covariance, lattice, kuhn, compliance) onto the helpers
 * below; see tests/test_oracle_pins.py. The whole-frame composition is pinned
 * only through those components.
 *
 * Every simulation entry point is available in float (the GPU's precision,
 * used for bit-exact parity) and double (the drift reference).
 */
#ifndef VSIM_ORACLE_H
#define VSIM_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#include "../include/vsim.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct vo_sim vo_sim;

/* precision: 32 or 64. */
int vo_create(const vsim_body_desc* bodies, uint32_t n, const vsim_tank* tank, int precision,
              vo_sim** out);
/* With flags = VSIM_CREATE_ISOLATED each body has its own contact grid and
   different bodies never touch (vsim_create_ex). */
int vo_create_ex(const vsim_body_desc* bodies, uint32_t n, const vsim_tank* tank, int precision, uint32_t flags,
                 vo_sim** out);
void vo_destroy(vo_sim* s);
void vo_set_threads(int threads);
int vo_max_threads(void);

int vo_set_step_duration(vo_sim* s, double seconds);
int vo_set_gravity(vo_sim* s, const double g[3]);
int vo_set_contact(vo_sim* s, int enabled);
int vo_set_self_contact(vo_sim* s, int enabled);
int vo_set_iterations(vo_sim* s, uint32_t iterations);
int vo_set_material(vo_sim* s, uint32_t body, const vsim_material* m, uint32_t fields);

int vo_hold(vo_sim* s, const uint32_t* nodes, const float* offsets, uint32_t count);
int vo_release(vo_sim* s);
int vo_set_drive_law(vo_sim* s, int law);
int vo_set_drive_response_time(vo_sim* s, double seconds);
/* The drive uniforms for the next frame: target and its velocity. */
int vo_set_grab(vo_sim* s, const double target[3], const double velocity[3]);

int vo_dispatch(vo_sim* s, uint32_t steps);

uint32_t vo_node_count(const vo_sim* s);
uint32_t vo_cell_count(const vo_sim* s);
uint32_t vo_surface_count(const vo_sim* s);
uint32_t vo_body_node_offset(const vo_sim* s, uint32_t body);
int vo_get_state(const vo_sim* s, float* pos, float* prev, float* vel);
int vo_get_state_f64(const vo_sim* s, double* pos, double* prev, double* vel);
int vo_set_state(vo_sim* s, const float* pos, const float* prev, const float* vel);
int vo_inv_mass(const vo_sim* s, float* out);
/* Body `b`'s occupied cells, colour-grouped, and the count per colour. */
int vo_cells(const vo_sim* s, uint32_t b, uint32_t* cells, uint32_t color_counts[8]);
int vo_surface(const vo_sim* s, uint32_t* nodes, uint32_t* bodies);
/* Overlapping contact pairs (a < b) of the current positions; returns the
   total, writes at most `capacity`. */
size_t vo_contact_pairs(const vo_sim* s, uint32_t* pairs, size_t capacity);
/* Grid layout the contact constraint uses: origin, bucket size, dims. */
int vo_contact_grid(const vo_sim* s, double origin[3], double* bucket, uint32_t dims[3]);

/* Splats of body `b` at the live positions (sample.wgsl:40-80,
   covariance.wgsl:30-42); depth keys as the library defines them. */
int vo_splat_deform(const vo_sim* s, uint32_t b, const float* means, const float* quats,
                    const float* scales, uint32_t n, const float view_dir[3], float* out_means,
                    float* out_cov6, uint32_t* keys);
/* Permutation sorting keys ascending, ties by index (std::stable_sort). */
void vo_stable_sort_u32(const uint32_t* keys, uint32_t n, uint32_t key_bits, uint32_t* order);

/* ---- known-answer helpers, double precision -------------------------- */

/* Kuhn tetrahedra (kuhn.js:28-35) and their rest shape inverses for a
   cell of edge h, column-major. */
void vo_kuhn_tets(uint32_t out[24]);
void vo_kuhn_rest_inverses(double h, double out[54]);
void vo_kuhn_rest_shapes(double h, double out[54]);
/* One tetrahedron's coupled projection (project.wgsl:90-152 with
   xpbdCouple.wgsl:58-71). p, prev: 4 x xyz. Compliances already over dt^2. */
void vo_project_tet_f64(const double* p, const double* prev, const double* w, const double* B,
                        double alpha_dev, double alpha_hyd, double gamma, double relax,
                        double* out);
/* A free tetrahedron run for `substeps` (predict, project, velocity), no
   gravity, no damping; the harness of elastic.test.js:253-264. */
void vo_run_free_tet_f64(double* p, const double* w, const double* B, double alpha_dev,
                         double alpha_hyd, double gamma, double relax, double dt,
                         uint32_t substeps);
/* Constraint values and gradients of one tetrahedron. */
void vo_tet_constraints_f64(const double* p, const double* B, double gamma, double* c_dev,
                            double* c_hyd, double* g_dev, double* g_hyd);
/* One contact's correction for `me` (collide.wgsl:70-118). Each node:
   position[3], previous[3], inv_mass, radius, friction. `me_index` and
   `mate_index` only orient the coincident case. Returns 0 when no overlap. */
int vo_resolve_pair_f64(const double* me, const double* mate, uint32_t me_index,
                        uint32_t mate_index, double out[3]);
/* Drive laws (driveHard.wgsl:15-35, driveCompliant.wgsl:24-41). */
void vo_drive_hard_f64(const double here[3], const double goal[3], const double velocity[3],
                       double dt, double position[3], double out_velocity[3]);
void vo_drive_compliant_f64(const double p[3], const double goal[3], double dt,
                            double response_time, double out[3]);
/* Unilateral length limit of one edge (project.wgsl:162-178). */
void vo_stretch_pair_f64(double a[3], double b[3], double wa, double wb, double maximum);
/* Tank plane with Coulomb friction (finalize.wgsl:29-42). */
void vo_resolve_plane_f64(const double p[3], const double prev[3], const double normal[3],
                          double depth, double friction, double out[3]);
/* Trilinear sampling of a deformed lattice (sample.wgsl:40-80). node_pos is
   xyz per node of one body. */
void vo_deformation_at_f64(const double* node_pos, const uint32_t node_dims[3],
                           const uint32_t cell_dims[3], const double origin[3], double h,
                           const double rest[3], double position[3], double gradient[9]);
/* Sigma' = (F R S)(F R S)^T, column-major 3x3 out (covariance.wgsl:30-42). */
void vo_deformed_covariance_f64(const double gradient[9], const double quat[4],
                                const double scale[3], double out[9]);
/* A covariance (xx, xy, xz, yy, yz, zz) as a unit quaternion xyzw and three
   axis lengths (ellipsoid.wgsl:20-91), in double and, for n covariances, in
   float as the GPU evaluates it. */
void vo_ellipsoid_axes_f64(const double cov6[6], double rotation[4], double scale[3]);
void vo_ellipsoid_axes_f32(const float* cov6, uint32_t n, float* rotation, float* scale);
/* 28 stretch edges: corner a, corner b, unit rest length (stretch.js:5-7). */
void vo_stretch_edges(double out[84]);
/* Grid layout of broadphase.js:46-58 for a bucket size. */
void vo_broadphase_grid(const double min[3], const double max[3], double bucket_size,
                        double origin[3], double* edge, uint32_t dims[3]);
uint32_t vo_bucket_of(const double origin[3], double bucket, const uint32_t dims[3],
                      const double point[3]);
/* Boundary nodes of a lattice (lattice.js:128-158). Returns the count. */
uint32_t vo_surface_nodes(const uint32_t cell_dims[3], const uint8_t* occupancy, uint32_t* out);

#ifdef __cplusplus
}
#endif

#endif
