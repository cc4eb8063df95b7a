/*
 * ORACLE -- test infrastructure, not product code.  CPU restatement of
 * jijn/phasefield_coarsening phasefield.c's explicit step; see
 * ppf_oracle.c for the line-by-line mapping.  Only tests/, the smoke check
 * and bench.py's CPU baseline use it.
 */
#ifndef PPF_ORACLE_H
#define PPF_ORACLE_H

#include <stdint.h>

#include "../include/ppf.h"

#ifdef __cplusplus
extern "C" {
#endif

/* phasefield.c:85-97 */
void ppf_oracle_derive(const ppf_params *p, ppf_derived *d);

/* Run `nsteps` iterations of the reference loop body (BC fill + sweep) on
 * interior arrays (nz*ny*nx, C order), in place.  Iterations with index
 * >= n_iter_init use the c-only sweep (phasefield.c:214-218).  sums (may
 * be NULL) receives sum dc^2, sum detaS^2, sum detaL^2 of the last step. */
int ppf_oracle_run(int nz, int ny, int nx, const ppf_params *p, int bc, int64_t nsteps,
                   int64_t n_iter_init, double *etaS, double *etaL, double *c, double sums[3]);

/* mass, solid, solid_cells, free energy, non-finite cells */
int ppf_oracle_observe(int nz, int ny, int nx, const ppf_params *p, int bc, const double *etaS,
                       const double *etaL, const double *c, double out[5]);

/* particles of etaS > thr: count, sum of equivalent radii, solid cells,
 * largest particle, solid/liquid faces; volumes by smallest cell index */
int ppf_oracle_particles(int nz, int ny, int nx, int bc, const double *etaS, double thr, double out[5],
                         int64_t *volumes, int64_t cap);

#ifdef __cplusplus
}
#endif
#endif
