/*
 * oracle.h -- CPU restatement of FJSPH's WCSPH hot path.  TEST INFRASTRUCTURE ONLY.
 *
 * This is the parity checker for the GB300 library and the timed CPU baseline.  It restates, in
 * FP64 with serial semantics, the reference functions named beside each entry point.  Nothing in
 * the product library may link or call it.
 *
 * Parity status: UNPINNED.  The reference ships no golden vectors and cannot be built here (its
 * Eigen / nanoflann / HDF5 / TECIO / NetCDF dependencies are not vendored).  The restatement is
 * checked against hand-derived known answers of the reference formulas and against the analytic
 * curves shipped with the reference examples (hydrostatic column).
 */
#ifndef FJSPH_ORACLE_H
#define FJSPH_ORACLE_H

#include "../include/fjsph_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_sim orc_sim;

orc_sim *orc_create(const fjsph_settings *s);
void orc_destroy(orc_sim *o);
void orc_set_settings(orc_sim *o, const fjsph_settings *s);
void orc_get_settings(orc_sim *o, fjsph_settings *s);
int orc_set_limits(orc_sim *o, const fjsph_block *blocks, int32_t nblocks, int64_t n_bound_blocks);
int orc_set_inlet(orc_sim *o, const fjsph_inlet *inlet);
int orc_get_inlet(orc_sim *o, fjsph_inlet *inlet);
int orc_get_limits(orc_sim *o, fjsph_block *blocks, int32_t max_blocks, int32_t *nblocks);
int orc_update_counts(orc_sim *o, int64_t *deleted);
int orc_set_state(orc_sim *o, int32_t which, const fjsph_state_view *st);
int orc_get_state(orc_sim *o, int32_t which, fjsph_state_view *st);
int64_t orc_particle_count(orc_sim *o);
void orc_set_threads(int32_t n);

int64_t orc_update_neighbours(orc_sim *o);                       /* Neighbours.cpp:7-47   */
void orc_neighbours_export(orc_sim *o, int64_t *off, int64_t *idx, double *d2);
double orc_dsph_prestep(orc_sim *o);                             /* Shifting.cpp:12-123   */
void orc_get_aero_velocity(orc_sim *o);                          /* Resid.cpp:569-611     */
void orc_detect_surface(orc_sim *o);                             /* Geometry.cpp:14-280   */
void orc_dissipation_terms(orc_sim *o);                          /* Shifting.cpp:126-186  */
void orc_particle_shift(orc_sim *o);                             /* Shifting.cpp:189-290  */
void orc_check_pipe_outlet(orc_sim *o);                          /* Containment.cpp:822   */
void orc_get_boundary_pressure(orc_sim *o);                      /* Resid.cpp:21-76       */
void orc_boundary_ghost(orc_sim *o, int32_t *near_inlet);        /* Resid.cpp:122-160     */
void orc_boundary_dbc(orc_sim *o);                               /* Resid.cpp:78-117      */
void orc_set_no_slip(orc_sim *o);                                /* Resid.cpp:162-186     */
void orc_get_acc_and_rrho(orc_sim *o, double npd);               /* Resid.cpp:426-469     */
double orc_find_timestep(orc_sim *o);                            /* Integration.cpp:370   */
double orc_get_first_rk(orc_sim *o, double npd);                 /* Runge_Kutta.cpp:462   */
double orc_runge_kutta4(orc_sim *o, double npd, double logbase); /* Runge_Kutta.cpp:480   */
void orc_nb_iter(orc_sim *o, double npd);                        /* Newmark_Beta.cpp:54   */
double orc_newmark_beta(orc_sim *o, double npd, double *logbase, int32_t *iteration);
double orc_integrate_no_update(orc_sim *o);                      /* Integration.cpp:27    */
double orc_integrate(orc_sim *o);                                /* Integration.cpp:233   */
void orc_step_report(orc_sim *o, double *out5);

/* Small known-answer helpers exposed for tests. */
double orc_kernel(double r, double H, double W_correc, int32_t cubic);
void orc_gradk(const double *Rij, double r, double H, double W_correc, int32_t cubic, int32_t dim, double *out);
double orc_min_eig(const double *A, int32_t dim);
int32_t orc_qr_inverse(const double *A, int32_t dim, double *inv);
double orc_get_cd(double Re);
/* vortex-lattice air source (VLM.cpp): setup returns the panel count (< 0 on a bad wing or a
 * singular influence matrix) */
int orc_vlm_setup(orc_sim *o, const fjsph_vlm *v);
int orc_air_power_law(orc_sim *o, const double *params4);
int orc_mesh_set(orc_sim *o, const fjsph_mesh *m);
int orc_vlm_panels(orc_sim *o, double *gamma, double *abc);
void orc_vlm_velocity(orc_sim *o, int64_t n, const double *pos, double *vel);

#ifdef __cplusplus
}
#endif

#endif
