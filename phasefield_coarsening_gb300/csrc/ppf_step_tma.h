// ppf_step_tma.h -- launcher of the TMA-fed fused step (ppf_step_tma.cuh).
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include "ppf_internal.h"

namespace ppf {

// One domain of an ensemble, as the fused step reads it from device memory
// (the TMA descriptors are used from there directly).
struct alignas(128) DomainDesc {
    CUtensorMap maps[2][3];   // [buffer][etaS, etaL, c]
    Geom g;
    void *fld[2][3];          // [buffer][etaS, etaL, c]
    int ntx, nty;             // tiles in x and y
    int nfx, nfy;             // whole tiles (inside the domain) in x and y
    int zc, nc;               // z planes per work item, items per tile column
    int item0[3], nitems[3];  // first work item and count of this domain in the ensemble's launch
                              // over edge tiles [0], over whole tiles [1], over every tile [2]
};

// Launch choices of the fused step that the autotuner may change.
struct StepTune {
    int grid;   // persistent CTAs
    int zc;     // z planes per work item
    int roll;   // 3: plane body unrolled three times; 1: one copy
    int pdl;    // 1: consecutive launches overlap by programmatic dependent launch
    int sched;  // 1: CTAs take work items from a global counter; 0: round-robin
    int zc2;    // > 0 (and < zc): the top `tail` planes are cut into chunks of zc2
    int tail;
    int split;  // 1: whole tiles and edge tiles as two overlapping launches; 0: one launch
    int tile;   // tile shape (step_tile); FP32 has two, FP64 one
};

// Tensor map of one padded field (3-D: x pitch, ny+2 rows, nz+2 planes)
// with the box of tile shape `tile`; 0 on success.
template <typename T>
int make_field_map(const Geom &g, const T *base, CUtensorMap *map, int tile);

// Persistent grid size (occupancy x SMs, capped by the work) and the z
// chunk length of a work item, for the first tile shape; < 0 on error.
template <typename T>
int tma_grid(const Geom &g, int num_sms, int *zc);

// Grid for a launch choice (occupancy x SMs, capped by its work items).
template <typename T>
int tma_grid_for(const Geom &g, int num_sms, const StepTune &t);

// One fused step.  maps = {etaS, etaL, c} of the input state; eqA selects
// the specialisation for AS == AL (mu needs no reciprocal); `partials`
// (nullable) receives 3 doubles per work item (tma_items of them); `err` is
// a device word that a CTA sets when an mbarrier wait exceeds limit_ns.
// inject_stall != 0 is a test hook that makes one wait per CTA run out.
// `sched` points to the step's two scheduler word pairs (four ints, zero
// before the first launch; every launch leaves them zero), used when
// tune.sched is set; steps that share them must be ordered on one stream.
template <typename T>
cudaError_t launch_step_tma(const Geom &g, const Coef<T> &k, const CUtensorMap *maps, Fields<T> out, bool c_only,
                            bool eqA, double *partials, const StepTune &tune, int *err, unsigned long long limit_ns,
                            int inject_stall, int *sched, cudaStream_t s);

// Work items of one single-domain step with the launch choice's z split.
template <typename T>
int64_t tma_items(const Geom &g, const StepTune &t);

// Tile (x, y) of tile shape `tile` of the fused step, and the number of
// tile shapes of the precision.
template <typename T>
void step_tile(int *tx, int *ty, int tile);
template <typename T>
int step_tile_shapes();

// Persistent grid of the ensemble step for `items` work items of tile
// shape `tile` (occupancy x SMs, capped).
template <typename T>
int tma_grid_items(int64_t items, int num_sms, int tile);

// One fused step of every domain of an ensemble: reads buffer `parity` of
// each domain and writes buffer 1-parity, as one launch over every tile
// (items[2] work items), or with `split` a launch over the whole tiles
// (items[1]) and one over the edge tiles (items[0]).  `partials` (nullable)
// receives 3 doubles per work item (the last-step increment sums; with the
// split the whole tiles' first); `sched` (nullable) as for launch_step_tma.
template <typename T>
cudaError_t launch_step_multi(const DomainDesc *table, int ndom, const int *items, const Coef<T> &k, bool c_only,
                              bool eqA, int parity, double *partials, int grid, int roll, bool pdl, bool split,
                              int tile, int *err, unsigned long long limit_ns, int *sched, cudaStream_t s);

}  // namespace ppf
