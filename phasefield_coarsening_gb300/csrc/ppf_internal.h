// ppf_internal.h -- device data layout and kernel launchers shared by the
// C-ABI translation units.  Not part of the public interface (include/ppf.h).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace ppf {

// HBM layout of one field: the reference's ghosted array
// double[NI+2][NJ+2][NK+2] (phasefield.c:67-70), with the x rows padded so
// that every row starts on a 32-byte sector and the interior x=0 does too:
//   storage(x, y, z) = (z+1)*PS + (y+1)*P + xoff + x,   x,y,z in [-1, n]
// xoff = 32 bytes / sizeof(T); P = row pitch, a multiple of 32 bytes with
// room for the ghost column x = nx.  Face ghosts hold the boundary
// condition for the next step; edges and corners are never read.
struct Geom {
    int nx, ny, nz;
    int xoff;
    int bc;
    int64_t P, PS, total;
    __host__ __device__ __forceinline__ int64_t at(int x, int y, int z) const {
        return (int64_t)(z + 1) * PS + (int64_t)(y + 1) * P + (int64_t)(x + xoff);
    }
};

template <typename T>
Geom make_geom(int nz, int ny, int nx, int bc) {
    Geom g;
    g.nx = nx; g.ny = ny; g.nz = nz; g.bc = bc;
    const int per32 = 32 / (int)sizeof(T);
    g.xoff = per32;
    g.P = ((int64_t)(g.xoff + nx + 1) + per32 - 1) / per32 * per32;
    g.PS = g.P * (ny + 2);
    g.total = g.PS * (nz + 2);
    return g;
}

// Loop-invariant coefficients of the step, folded on the host in double
// from the constants block (phasefield.c:76-97) and sweep_fields' own
// invariants (tmp1..tmp6, :322-323, :337-339), then cast once to the
// step's precision.  The folding rests on two exact identities of the KKS
// construction of :351-359: with mu = AS AL/(AS+(AL-AS)hS) (c-cL0+(cL0-cS0)hS)
// the phase compositions satisfy AS (cS-cS0) = AL (cL-cL0) = mu, hence
//   fS - fL - mu (cS - cL) = (CS-CL) - mu ((cS0-cL0) + (1/AS-1/AL)/2 mu),
// and detaS, detaL, dc of :360-384 are rearranged with tmp1, tmp3 absorbed.
template <typename T>
struct Coef {
    T AS, dA, AsAl;   // AS, AL-AS, AS*AL: mu = AsAl/(AS+dA h) (c-cL0+dc0 h)
    T A;              // AS (= AL when eqA): mu = A (c-cL0+dc0 h)
    T cL0, dc0;       // cL0, cL0-cS0
    T Mt0, Mt1;       // tmp3*ML, tmp3*(MS-ML): M' = tmp3 M = Mt0 + Mt1 h
    T dC, q1, q2;     // CS-CL, cS0-cL0, (1/AS-1/AL)/2: driving force D = dC - mu (q1 + q2 mu)
    T dm2;            // 2 tmp1: tmp1 dmu = dm2 etaS etaL / (etaS^2+etaL^2)^2 D
    T mt, tg, kt;     // tmp1 m, 2 gamma, tmp1 kappa h2
};

// The same coefficients in double, plus what the observables need.
struct CoefD {
    double AS, AL, dA, cS0, cL0, CS, CL, tmp2, m, gamma, kappa_h2_half, vol;
};

template <typename T>
struct Fields {
    T *eS, *eL, *c;
};

// Pack/unpack between compact double arrays [z][y][x] and the padded
// layout; pack also writes the face ghosts (the BC fill of :207-211).
template <typename T>
cudaError_t launch_pack(const Geom &g, const double *src3, Fields<T> dst, cudaStream_t s);
template <typename T>
cudaError_t launch_unpack(const Geom &g, Fields<const T> src, double *dst3, cudaStream_t s);

// One domain of a batched pack / unpack (device table): its geometry, its
// compact float64 staging array (3 fields), its two state buffers and its
// device results (the increment sums a fresh upload clears).
struct IoDesc {
    Geom g;
    double *staging;
    void *fld[2][3];
    double *dres;
};

// Pack every domain's staging into its buffer 0 (clearing its increment
// sums), or unpack every domain's buffer `buf` into its staging: one launch
// for `n` domains (grid y = domain), the largest holding max_cells cells.
template <typename T>
cudaError_t launch_pack_multi(const IoDesc *table, int n, int64_t max_cells, cudaStream_t s);
template <typename T>
cudaError_t launch_unpack_multi(const IoDesc *table, int n, int64_t max_cells, int buf, cudaStream_t s);

// Observables of a state: per-CTA partial sums of
// {mass, solid, solid_cells, free energy, nonfinite} into partials[5*b+i].
template <typename T>
cudaError_t launch_observe(const Geom &g, const CoefD &k, Fields<const T> f, double *partials,
                           int nblocks, cudaStream_t s);

// Record `msg` as the calling thread's ppf_last_error() text; returns code.
int set_last_error(int code, const char *msg);

// Deterministic final sum: out[i] = sum_b partials[stride*b + i] for
// i < nvals (fixed order, one CTA).
cudaError_t launch_final_sum(const double *partials, int nblocks, int stride, int nvals, double *out,
                             cudaStream_t s);

}  // namespace ppf
