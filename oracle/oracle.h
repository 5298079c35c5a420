/* oracle.h - TEST INFRASTRUCTURE ONLY: C interface of the serial restatement
 * of din-mol-Li's hot path (dana_oracle.cpp).  Loaded by tests/, the smoke
 * check and bench.py's CPU-baseline leg; never by the product. */
#ifndef DML_ORACLE_H
#define DML_ORACLE_H

#include <stdint.h>

#include "../include/dml.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_sim orc_sim;

/* Reference constants (src/dana.F90:12-25, 81-100, 113; src/Constants.F90:
 * 105-167) and the tests/ermak run values. */
static inline void dml_params_default_oracle(dml_params* p) {
  /* program dana: kB_ui = kB_eVK * eV_ui, eV_ui = 96.485 * 100 */
  const double eV_ui = 96.485 * 100.0;
  /* gems_constants: kB_ui = kB_ev * ev_ui, ev_ui = 1 / (axps_mxs^2 uma_kg joule_ev) */
  const double joule_ev = 1.0 / 1.60219e-19;
  const double ui_ev = 1.0e2 * 1.0e2 * 1.6605402e-27 * joule_ev;
  const double ev_ui = 1.0 / ui_ev;
  int i, j;
  p->box[0] = 100.0;
  p->box[1] = 100.0;
  p->box[2] = 200.0;
  p->z0 = 100.0;
  p->zmax = 200.0;
  p->z1 = 0.0;
  p->h = 1.e-2;
  p->gamma = 1.0;
  p->temp = 300.0;
  p->kb_driver = 8.617330350e-5 * eV_ui;
  p->kb_module = 8.617385e-05 * ev_ui;
  for (i = 0; i < 3; ++i)
    for (j = 0; j < 3; ++j) {
      p->eps[i][j] = 0.0;
      p->r0[i][j] = 0.0;
    }
  p->r0[1][0] = 3.5;
  p->r0[0][1] = 3.5;
  p->eps[0][0] = 2313.6;
  p->r0[0][0] = 3.2;
  p->eps[2][2] = 121.0;
  p->r0[2][2] = 3.61;
  p->eps[0][2] = 529.1;
  p->eps[2][0] = 529.1;
  p->r0[0][2] = 1.564;
  p->r0[2][0] = 1.564;
  p->mass[0] = p->mass[1] = p->mass[2] = 6.94;
  p->rc = 3.2;
  p->skin = 10.0;
  p->prob = 1.0;
  p->dif_sc = 250.0;
  p->dif_sei = 250.0;
  p->dif_switch_z = 80.0;
  p->tau = 0.1;
  p->act = 0.0;
  p->nadj = 0;
  p->integrator = DML_INTEGRATOR_ERMAK;
  p->reservoir = DML_RESERVOIR_PISTON;
  p->precision = DML_PRECISION_FP64;
  p->mnb = 10000;
  p->capacity = 0;
  p->max_passes = 64;
  p->event_cap = 64;
  p->seed = 0;
}

orc_sim* orc_create(const dml_params* p, int32_t rng_mode, int32_t idum);
void orc_destroy(orc_sim* o);
int orc_set_atoms(orc_sim* o, const dml_atoms* a);
int orc_setup(orc_sim* o);
int orc_step(orc_sim* o, int64_t nsteps);
int orc_test_update(orc_sim* o, int32_t* rebuilt);
int orc_force(orc_sim* o);
int orc_ermak_a(orc_sim* o, int64_t step);
int orc_ermak_b(orc_sim* o);
int orc_brownian(orc_sim* o, int64_t step);
int orc_overlap_moveback(orc_sim* o, int64_t step);
int orc_capture_commit(orc_sim* o, int32_t* n_new);
int orc_gcmc(orc_sim* o, int64_t step);
int orc_calc_rho(orc_sim* o, double* rho);
int orc_set_chunk(orc_sim* o, int32_t n, const double* pos, const int32_t* z, double dist);
int orc_bloques(orc_sim* o);
int orc_piston(orc_sim* o);
int orc_get_atoms(orc_sim* o, dml_atoms* a);
int orc_get_neighbors(orc_sim* o, int32_t* n_ref, int32_t* nn, int32_t* list, int32_t ld);
int orc_get_counters(orc_sim* o, dml_counters* c);
int orc_reset_counters(orc_sim* o);
int orc_salida(orc_sim* o, dml_observables* out);
const char* orc_errmsg(orc_sim* o);
void orc_set_step(orc_sim* o, int64_t step);
int orc_run_reference_case(const char* dir, int32_t max_n, int32_t* n_out, double* pos_out,
                           int32_t* z_out, double* zmax_out, int64_t* counters_out);

#ifdef __cplusplus
}
#endif

#endif
