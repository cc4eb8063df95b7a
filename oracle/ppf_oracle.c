/*
 * ORACLE -- test infrastructure, not product code.
 *
 * A plain-C restatement of the reference's explicit step, used only as the
 * oracle by tests/, by __graft_entry__.smoke() and by bench.py's CPU
 * baseline leg.  Nothing in the product links or calls it.
 *
 * It follows jijn/phasefield_coarsening phasefield.c line by line:
 *   constants            :76-97    -> ppf_oracle_derive
 *   array initialisation :156-167  -> oracle_alloc
 *   BC fill (serial)     :1112-1148 periodic, :1151-1189 no-flux -> bc_fill
 *   sweep_fields         :301-403  -> sweep_fields
 *   sweep_fields_c       :406-476  -> sweep_fields_c
 *   loop + error sums    :178-258  -> ppf_oracle_run
 * Arrays are ghosted [nz+2][ny+2][nx+2], index [z][y][x] (= [i][j][k] of
 * the reference, :53-56).  The only deviation from the reference program is
 * that the grid size, BC, dt and step counts are run-time arguments instead
 * of compile-time constants.  Loops carry OpenMP pragmas (no effect on the
 * arithmetic: every pass writes each cell from values the pass does not
 * write).
 *
 * The observables (ppf_oracle_observe) have no counterpart in the
 * reference; they define the solute mass, phase fraction and free energy
 * that the GPU reductions are checked against.
 */
#include "ppf_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#define IDX(i, j, k) (((size_t)(i) * (size_t)(NJ + 2) + (size_t)(j)) * (size_t)(NK + 2) + (size_t)(k))

void ppf_oracle_derive(const ppf_params *p, ppf_derived *d)
{
    /* phasefield.c:85 */
    d->ML = p->DL / p->AL;
    d->MS = p->DS / p->AS;
    /* :91-92 */
    d->h2 = 1.0 / (p->dx * p->dx);
    d->dt = p->dt > 0 ? p->dt : 0.125 * p->dx * p->dx / p->DL;
    /* :94-97 */
    d->l = p->l > 0 ? p->l : 7.0 * p->dx;
    d->m = 6.0 * p->sigma / d->l;
    d->kappa = 3 * 0.25 * p->sigma * d->l;
    d->L = 4.0 / 3.0 * d->m / d->kappa *
           (0.5 * (d->MS + d->ML) / ((p->cSeq - p->cLeq) * (p->cSeq - p->cLeq)));
    double D = p->DL > p->DS ? p->DL : p->DS;
    d->dt_limit = p->dx * p->dx / (6.0 * D);
}

typedef struct {
    int NI, NJ, NK;
    double *etaS, *detaS, *etaL, *detaL, *c, *dc, *hS, *mu, *M;
} ostate;

/* phasefield.c:156-167: every array starts at 1.0, the increments at 0. */
static int oracle_alloc(ostate *s, int nz, int ny, int nx)
{
    s->NI = nz; s->NJ = ny; s->NK = nx;
    size_t n = (size_t)(nz + 2) * (size_t)(ny + 2) * (size_t)(nx + 2);
    double **a[9] = {&s->etaS, &s->detaS, &s->etaL, &s->detaL, &s->c, &s->dc, &s->hS, &s->mu, &s->M};
    for (int f = 0; f < 9; ++f) {
        *a[f] = (double *)malloc(n * sizeof(double));
        if (!*a[f]) return -1;
    }
    for (size_t q = 0; q < n; ++q) {
        s->etaS[q] = 1.0; s->detaS[q] = 0.0;
        s->etaL[q] = 1.0; s->detaL[q] = 0.0;
        s->c[q] = 1.0;    s->dc[q] = 0.0;
        s->hS[q] = 1.0;   s->mu[q] = 1.0;   s->M[q] = 1.0;
    }
    return 0;
}

static void oracle_free(ostate *s)
{
    free(s->etaS); free(s->detaS); free(s->etaL); free(s->detaL);
    free(s->c); free(s->dc); free(s->hS); free(s->mu); free(s->M);
}

/* phasefield.c:1112-1148 (periodic) and :1151-1189 (no-flux): faces only,
 * edges and corners untouched. */
static void bc_fill(ostate *s, int bc)
{
    const int NI = s->NI, NJ = s->NJ, NK = s->NK;
    double *f3[3] = {s->etaS, s->etaL, s->c};
    for (int f = 0; f < 3; ++f) {
        double *u = f3[f];
        for (int j = 1; j <= NJ; j++)
            for (int k = 1; k <= NK; k++) {
                u[IDX(0, j, k)] = bc == PPF_BC_PERIODIC ? u[IDX(NI, j, k)] : u[IDX(1, j, k)];
                u[IDX(NI + 1, j, k)] = bc == PPF_BC_PERIODIC ? u[IDX(1, j, k)] : u[IDX(NI, j, k)];
            }
        for (int i = 1; i <= NI; i++)
            for (int k = 1; k <= NK; k++) {
                u[IDX(i, 0, k)] = bc == PPF_BC_PERIODIC ? u[IDX(i, NJ, k)] : u[IDX(i, 1, k)];
                u[IDX(i, NJ + 1, k)] = bc == PPF_BC_PERIODIC ? u[IDX(i, 1, k)] : u[IDX(i, NJ, k)];
            }
        for (int i = 1; i <= NI; i++)
            for (int j = 1; j <= NJ; j++) {
                u[IDX(i, j, 0)] = bc == PPF_BC_PERIODIC ? u[IDX(i, j, NK)] : u[IDX(i, j, 1)];
                u[IDX(i, j, NK + 1)] = bc == PPF_BC_PERIODIC ? u[IDX(i, j, 1)] : u[IDX(i, j, NK)];
            }
    }
}

/* pass A of sweep_fields / sweep_fields_c, phasefield.c:322-335 / :422-435 */
static void pass_a(ostate *s, const ppf_params *p, const ppf_derived *d)
{
    const int NI = s->NI, NJ = s->NJ, NK = s->NK;
    const double AS = p->AS, AL = p->AL, cL0 = p->cL0, cS0 = p->cS0;
    const double MS = d->MS, ML = d->ML;
    const double tmp5 = AS * AL;
    const double tmp6 = cL0 - cS0;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < NI + 2; i++)
        for (int j = 0; j < NJ + 2; j++)
            for (int k = 0; k < NK + 2; k++) {
                size_t q = IDX(i, j, k);
                s->hS[q] = s->etaS[q] * s->etaS[q] / (s->etaS[q] * s->etaS[q] + s->etaL[q] * s->etaL[q]);
                s->mu[q] = tmp5 / (AS + (AL - AS) * s->hS[q]) * (s->c[q] - cL0 + tmp6 * s->hS[q]);
                s->M[q] = ML + (MS - ML) * s->hS[q];
            }
}

/* the solute flux divergence of phasefield.c:374-384 / :449-459 */
static inline double dc_of(const ostate *s, int i, int j, int k, double tmp3)
{
    const int NJ = s->NJ, NK = s->NK;
    const double *M = s->M, *mu = s->mu;
    return tmp3 * (M[IDX(i + 1, j, k)] * (mu[IDX(i + 1, j, k)] - mu[IDX(i, j, k)]) -
                   M[IDX(i - 1, j, k)] * (mu[IDX(i, j, k)] - mu[IDX(i - 1, j, k)]) +
                   M[IDX(i, j + 1, k)] * (mu[IDX(i, j + 1, k)] - mu[IDX(i, j, k)]) -
                   M[IDX(i, j - 1, k)] * (mu[IDX(i, j, k)] - mu[IDX(i, j - 1, k)]) +
                   M[IDX(i, j, k + 1)] * (mu[IDX(i, j, k + 1)] - mu[IDX(i, j, k)]) -
                   M[IDX(i, j, k - 1)] * (mu[IDX(i, j, k)] - mu[IDX(i, j, k - 1)]) +
                   M[IDX(i, j, k)] * (mu[IDX(i + 1, j, k)] + mu[IDX(i - 1, j, k)] +
                                      mu[IDX(i, j + 1, k)] + mu[IDX(i, j - 1, k)] +
                                      mu[IDX(i, j, k + 1)] + mu[IDX(i, j, k - 1)] - 6.0 * mu[IDX(i, j, k)]));
}

/* sweep_fields, phasefield.c:301-403 */
static void sweep_fields(ostate *s, const ppf_params *p, const ppf_derived *d)
{
    const int NI = s->NI, NJ = s->NJ, NK = s->NK;
    const double AS = p->AS, AL = p->AL, cL0 = p->cL0, cS0 = p->cS0, CS = p->CS, CL = p->CL;
    const double L = d->L, dt = d->dt, h2 = d->h2, m = d->m, gamma = p->gamma, kappa = d->kappa;
    pass_a(s, p, d);
    const double tmp1 = -1.0 * L * dt;     /* :337 */
    const double tmp2 = (AS * cS0 - AL * cL0);
    const double tmp3 = dt * 0.5 * h2;
    double *etaS = s->etaS, *etaL = s->etaL;
#pragma omp parallel for schedule(static)
    for (int i = 1; i <= NI; i++)
        for (int j = 1; j <= NJ; j++)
            for (int k = 1; k <= NK; k++) {
                size_t q = IDX(i, j, k);
                double hS = s->hS[q], c = s->c[q], mu = s->mu[q];
                double eS = etaS[q], eL = etaL[q];
                double tmp4 = 1.0 / (AS + (AL - AS) * hS);                 /* :351 */
                double cS = tmp4 * (AL * c + (1.0 - hS) * tmp2);
                double cL = tmp4 * (AS * c - hS * tmp2);
                double fS = 0.5 * AS * (cS - cS0) * (cS - cS0) + CS;
                double fL = 0.5 * AL * (cL - cL0) * (cL - cL0) + CL;
                double dmu = 2.0 * (eS * eL) / ((eS * eS + eL * eL) * (eS * eS + eL * eL)) *
                             (fS - fL - mu * (cS - cL));                   /* :356-359 */
                s->detaS[q] = tmp1 * (m * eS * (eS * eS - 1.0 + 2.0 * gamma * eL * eL) -
                                      kappa * h2 * (etaS[IDX(i + 1, j, k)] + etaS[IDX(i - 1, j, k)] +
                                                    etaS[IDX(i, j + 1, k)] + etaS[IDX(i, j - 1, k)] +
                                                    etaS[IDX(i, j, k + 1)] + etaS[IDX(i, j, k - 1)] - 6.0 * eS) +
                                      eL * dmu);                           /* :360-366 */
                s->detaL[q] = tmp1 * (m * eL * (eL * eL - 1.0 + 2.0 * gamma * eS * eS) -
                                      kappa * h2 * (etaL[IDX(i + 1, j, k)] + etaL[IDX(i - 1, j, k)] +
                                                    etaL[IDX(i, j + 1, k)] + etaL[IDX(i, j - 1, k)] +
                                                    etaL[IDX(i, j, k + 1)] + etaL[IDX(i, j, k - 1)] - 6.0 * eL) -
                                      eS * dmu);                           /* :367-373 */
                s->dc[q] = dc_of(s, i, j, k, tmp3);                        /* :374-384 */
            }
    /* :393-401: the update runs over the ghosts too, whose increments stay 0 */
    size_t n = (size_t)(NI + 2) * (size_t)(NJ + 2) * (size_t)(NK + 2);
#pragma omp parallel for schedule(static)
    for (size_t q = 0; q < n; ++q) {
        etaS[q] = etaS[q] + s->detaS[q];
        etaL[q] = etaL[q] + s->detaL[q];
        s->c[q] = s->c[q] + s->dc[q];
    }
}

/* sweep_fields_c, phasefield.c:406-476 */
static void sweep_fields_c(ostate *s, const ppf_params *p, const ppf_derived *d)
{
    const int NI = s->NI, NJ = s->NJ, NK = s->NK;
    pass_a(s, p, d);
    const double tmp3 = d->dt * 0.5 * d->h2;   /* :437 */
#pragma omp parallel for schedule(static)
    for (int i = 1; i <= NI; i++)
        for (int j = 1; j <= NJ; j++)
            for (int k = 1; k <= NK; k++) s->dc[IDX(i, j, k)] = dc_of(s, i, j, k, tmp3);
    size_t n = (size_t)(NI + 2) * (size_t)(NJ + 2) * (size_t)(NK + 2);
#pragma omp parallel for schedule(static)
    for (size_t q = 0; q < n; ++q) s->c[q] = s->c[q] + s->dc[q];
}

static void copy_in(ostate *s, const double *src, double *dst)
{
    const int NI = s->NI, NJ = s->NJ, NK = s->NK;
    for (int i = 1; i <= NI; i++)
        for (int j = 1; j <= NJ; j++)
            memcpy(dst + IDX(i, j, 1), src + ((size_t)(i - 1) * NJ + (j - 1)) * NK, (size_t)NK * sizeof(double));
}

static void copy_out(ostate *s, const double *src, double *dst)
{
    const int NI = s->NI, NJ = s->NJ, NK = s->NK;
    for (int i = 1; i <= NI; i++)
        for (int j = 1; j <= NJ; j++)
            memcpy(dst + ((size_t)(i - 1) * NJ + (j - 1)) * NK, src + IDX(i, j, 1), (size_t)NK * sizeof(double));
}

int ppf_oracle_run(int nz, int ny, int nx, const ppf_params *p, int bc, int64_t nsteps,
                   int64_t n_iter_init, double *etaS, double *etaL, double *c, double sums[3])
{
    if (nz < 1 || ny < 1 || nx < 1 || !p || !etaS || !etaL || !c || nsteps < 0) return -1;
    if (bc != PPF_BC_PERIODIC && bc != PPF_BC_NOFLUX) return -1;
    ppf_derived d;
    ppf_oracle_derive(p, &d);
    ostate s;
    memset(&s, 0, sizeof s);
    if (oracle_alloc(&s, nz, ny, nx)) { oracle_free(&s); return -2; }
    copy_in(&s, etaS, s.etaS);
    copy_in(&s, etaL, s.etaL);
    copy_in(&s, c, s.c);
    /* phasefield.c:179-218: BC fill, then the full or the c-only sweep */
    for (int64_t it = 0; it < nsteps; ++it) {
        bc_fill(&s, bc);
        if (it < n_iter_init) sweep_fields(&s, p, &d);
        else sweep_fields_c(&s, p, &d);
    }
    /* :228-238: interior sums of the last increments */
    if (sums) {
        const int NI = s.NI, NJ = s.NJ, NK = s.NK;
        double e = 0, e3 = 0, e4 = 0;
        for (int i = 1; i <= NI; i++)
            for (int j = 1; j <= NJ; j++)
                for (int k = 1; k <= NK; k++) {
                    size_t q = IDX(i, j, k);
                    e += s.dc[q] * s.dc[q];
                    e3 += s.detaS[q] * s.detaS[q];
                    e4 += s.detaL[q] * s.detaL[q];
                }
        sums[0] = e; sums[1] = e3; sums[2] = e4;
    }
    copy_out(&s, s.etaS, etaS);
    copy_out(&s, s.etaL, etaL);
    copy_out(&s, s.c, c);
    oracle_free(&s);
    return 0;
}

/* Observables of a state (no counterpart in the reference):
 *   out[0] mass        sum c
 *   out[1] solid       sum hS,  hS = etaS^2/(etaS^2+etaL^2)           (:328-330)
 *   out[2] solid_cells count of etaS > 0.5
 *   out[3] free energy sum over cells of dx^3 * (
 *            m (etaS^4/4 - etaS^2/2 + etaL^4/4 - etaL^2/2 + gamma etaS^2 etaL^2 + 1/4)
 *          + kappa/2 h2 sum_{d=x,y,z} [(etaS(+d)-etaS)^2 + (etaL(+d)-etaL)^2]
 *          + hS fS(cS) + (1-hS) fL(cL) )
 *          with the KKS phase compositions cS, cL and parabolas fS, fL of
 *          :351-355; the +d neighbour of the last cell is its ghost
 *          (periodic wrap, or the cell itself for no-flux).  The variational
 *          derivative of this functional is the bracket of :360-373.
 *   out[4] cells with a non-finite value in any field */
int ppf_oracle_observe(int nz, int ny, int nx, const ppf_params *p, int bc, const double *etaS,
                       const double *etaL, const double *c, double out[5])
{
    if (nz < 1 || ny < 1 || nx < 1 || !p || !out) return -1;
    ppf_derived d;
    ppf_oracle_derive(p, &d);
    const double AS = p->AS, AL = p->AL, cL0 = p->cL0, cS0 = p->cS0, CS = p->CS, CL = p->CL;
    const double tmp2 = AS * cS0 - AL * cL0;
    const double vol = p->dx * p->dx * p->dx;
    double mass = 0, solid = 0, cnt = 0, F = 0, bad = 0;
#pragma omp parallel for schedule(static) reduction(+ : mass, solid, cnt, F, bad)
    for (int z = 0; z < nz; ++z)
        for (int y = 0; y < ny; ++y)
            for (int x = 0; x < nx; ++x) {
                size_t q = ((size_t)z * ny + y) * nx + x;
                double eS = etaS[q], eL = etaL[q], cc = c[q];
                if (!isfinite(eS) || !isfinite(eL) || !isfinite(cc)) { bad += 1; continue; }
                int xp = x + 1 < nx ? x + 1 : (bc == PPF_BC_PERIODIC ? 0 : x);
                int yp = y + 1 < ny ? y + 1 : (bc == PPF_BC_PERIODIC ? 0 : y);
                int zp = z + 1 < nz ? z + 1 : (bc == PPF_BC_PERIODIC ? 0 : z);
                size_t qx = ((size_t)z * ny + y) * nx + xp;
                size_t qy = ((size_t)z * ny + yp) * nx + x;
                size_t qz = ((size_t)zp * ny + y) * nx + x;
                double s2 = eS * eS + eL * eL;
                double h = eS * eS / s2;
                mass += cc;
                solid += h;
                cnt += eS > 0.5 ? 1.0 : 0.0;
                double f0 = eS * eS * eS * eS / 4 - eS * eS / 2 + eL * eL * eL * eL / 4 - eL * eL / 2 +
                            p->gamma * eS * eS * eL * eL + 0.25;
                double g = 0;
                g += (etaS[qx] - eS) * (etaS[qx] - eS) + (etaL[qx] - eL) * (etaL[qx] - eL);
                g += (etaS[qy] - eS) * (etaS[qy] - eS) + (etaL[qy] - eL) * (etaL[qy] - eL);
                g += (etaS[qz] - eS) * (etaS[qz] - eS) + (etaL[qz] - eL) * (etaL[qz] - eL);
                double tmp4 = 1.0 / (AS + (AL - AS) * h);
                double cS = tmp4 * (AL * cc + (1.0 - h) * tmp2);
                double cL = tmp4 * (AS * cc - h * tmp2);
                double fS = 0.5 * AS * (cS - cS0) * (cS - cS0) + CS;
                double fL = 0.5 * AL * (cL - cL0) * (cL - cL0) + CL;
                F += vol * (d.m * f0 + 0.5 * d.kappa * d.h2 * g + h * fS + (1.0 - h) * fL);
            }
    out[0] = mass; out[1] = solid; out[2] = cnt; out[3] = F; out[4] = bad;
    return 0;
}

/* Particle analysis (no counterpart in the reference): 6-connected
 * components of etaS > thr, wrapping across periodic faces.  out[0] count,
 * out[1] sum of equivalent radii (3V/4pi)^(1/3) (cells, dx = 1), out[2]
 * solid cells, out[3] largest particle (cells), out[4] solid/liquid faces.
 * volumes (may be NULL) receives up to cap particle volumes, ordered by
 * the smallest cell index of each particle. */
static int64_t uf_find(int64_t *p, int64_t i)
{
    while (p[i] != i) {
        p[i] = p[p[i]];
        i = p[i];
    }
    return i;
}

int ppf_oracle_particles(int nz, int ny, int nx, int bc, const double *etaS, double thr, double out[5],
                         int64_t *volumes, int64_t cap)
{
    if (nz < 1 || ny < 1 || nx < 1 || !etaS || !out) return -1;
    const int64_t n = (int64_t)nz * ny * nx;
    int64_t *p = (int64_t *)malloc((size_t)n * sizeof(int64_t));
    int64_t *v = (int64_t *)calloc((size_t)n, sizeof(int64_t));
    if (!p || !v) { free(p); free(v); return -2; }
    for (int64_t i = 0; i < n; ++i) p[i] = etaS[i] > thr ? i : -1;
    double faces = 0;
    for (int z = 0; z < nz; ++z)
        for (int y = 0; y < ny; ++y)
            for (int x = 0; x < nx; ++x) {
                const int64_t i = ((int64_t)z * ny + y) * nx + x;
                const int c[3][3] = {{x + 1, y, z}, {x, y + 1, z}, {x, y, z + 1}};
                const int lim[3] = {nx, ny, nz};
                for (int d = 0; d < 3; ++d) {
                    int q[3] = {c[d][0], c[d][1], c[d][2]};
                    if (q[d] == lim[d]) {
                        if (bc != PPF_BC_PERIODIC) continue;
                        q[d] = 0;
                    }
                    const int64_t j = ((int64_t)q[2] * ny + q[1]) * nx + q[0];
                    const int si = p[i] >= 0, sj = p[j] >= 0;
                    if (si != sj) faces += 1.0;
                    if (si && sj) {
                        int64_t a = uf_find(p, i), b = uf_find(p, j);
                        if (a != b) {
                            if (a < b) p[b] = a;
                            else p[a] = b;
                        }
                    }
                }
            }
    double cnt = 0, rsum = 0, solid = 0, vmax = 0;
    for (int64_t i = 0; i < n; ++i)
        if (p[i] >= 0) {
            v[uf_find(p, i)] += 1;
            solid += 1;
        }
    int64_t k = 0;
    for (int64_t i = 0; i < n; ++i)
        if (p[i] == i) {
            cnt += 1;
            rsum += cbrt(3.0 * (double)v[i] / (4.0 * 3.14159265358979323846));
            if ((double)v[i] > vmax) vmax = (double)v[i];
            if (volumes && k < cap) volumes[k] = v[i];
            ++k;
        }
    out[0] = cnt; out[1] = rsum; out[2] = solid; out[3] = vmax; out[4] = faces;
    free(p);
    free(v);
    return 0;
}
