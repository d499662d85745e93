/*
 * md_oracle.h -- CPU oracle for the short-range MD path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference
 * implementation's algorithm (LinkedCells binning, serial periodic halo, C08
 * cell-pair traversal with the VectorizedCellProcessor site-site bodies,
 * FullMolecule::calcFM, Leapfrog) used as the checker in tests/, by
 * __graft_entry__.smoke() and by bench.py's CPU baseline.  The product path
 * never links or calls it.  Its results are pinned against the reference's
 * own outputs in tests/golden/ (generated by tests/golden/make_golden.py).
 *
 * It shares the plain data structs of include/ls1gb300.h so that tests pass
 * identical inputs to the oracle and to the engine.
 */
#ifndef MD_ORACLE_H
#define MD_ORACLE_H

#include "../include/ls1gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_sys orc_sys;

orc_sys* orc_create(const md_config* cfg, const md_component* comps, int32_t ncomp, const double* mixing);
void orc_destroy(orc_sys* s);
int orc_set_threads(int32_t n);
int orc_set_molecules(orc_sys* s, int64_t n, const uint64_t* id, const int32_t* comp, const double* r,
                      const double* v, const double* q, const double* L);
int64_t orc_num_molecules(const orc_sys* s);
/* F, M, Vi (n x 3, molecule order; NULL: unchanged) */
int orc_set_forces(orc_sys* s, int64_t n, const double* F, const double* M, const double* Vi);
int orc_get_molecules(const orc_sys* s, int64_t n, uint64_t* id, int32_t* comp, double* r, double* v,
                      double* q, double* L, double* F, double* M, double* Vi);
/* wrap leavers (periodic dims), bin, build halo copies, build site caches */
int orc_rebin_and_halo(orc_sys* s, md_bin_stats* st);
int orc_get_cells(const orc_sys* s, int64_t n, int64_t* cell);
/* traversal + calcFM; kernel_calls receives the FlopCounter-style counts
 * including inner-halo duplicates (1 + 7 entries: molecule distances, kinds). */
int orc_forces(orc_sys* s, md_forces_out* out, double* kernel_calls);
int orc_pre(orc_sys* s, double dt);
int orc_post(orc_sys* s, double dt, md_kinetic_out* out);
int orc_run(orc_sys* s, double dt, int32_t nsteps, md_step_record* rec);
/* reduced memory mode (LeapfrogRMM + VCP1CLJRMM): forces with the velocity
 * kick v += dt_inv_m F, drift r += dt v, velocity sums v.v without the mass,
 * and whole steps */
int orc_rmm_forces(orc_sys* s, double dt_inv_m, md_forces_out* out);
int orc_rmm_positions(orc_sys* s, double dt);
int orc_rmm_velocities(const orc_sys* s, md_kinetic_out* out);
int orc_rmm_run(orc_sys* s, double dt, int32_t nsteps, md_step_record* rec);
/* global velocity-scaling thermostat (target <= 0: NVE), applied by orc_run */
int orc_set_thermostat(orc_sys* s, double target_temperature, int32_t explosion_heuristics);
int orc_thermostat(orc_sys* s, const md_kinetic_out* ko, double* beta_trans, double* beta_rot);
/* Homogeneous long-range correction (longRange/Homogeneous.cpp:22-146) */
int orc_longrange_homogeneous(const orc_sys* s, double* upot_corr, double* virial_corr);

#ifdef __cplusplus
}
#endif
#endif
