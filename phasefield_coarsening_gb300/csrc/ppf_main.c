/*
 * ppf_main.c -- the `ppf` program: drop-in for the reference's main
 * (jijn/phasefield_coarsening phasefield.c:73-269) with the time step on
 * the GPU through include/ppf.h.
 *
 *   ppf <file.h5> [options]
 *
 * Same contract as the reference:
 *   - reads /etaS, /etaL, /c (3-D float64, [z][y][x]) from <file.h5>
 *     (phasefield.c:996-1049); the grid size is the datasets' size;
 *   - job name = the file name with its last three characters (".h5")
 *     replaced by "_" (:117-121), printed as "The job name is %s";
 *   - iteration i (from 0) applies the BC and one sweep (:179-218); at
 *     i > 0 with i % n_save == 0 or i == n_iter_init it prints the interior
 *     sums "%ld: c=%10.4e; S=%10.4e; L=%10.4e\t" and
 *     "iter: %ld; err: %10.4e\n" on stderr, writes <job><k>.h5 (k = 1, 2,
 *     ...) holding etaS, etaL, c and prints that name on stdout
 *     (:221-256, :1193-1213);
 *   - the loop stops after n_iter iterations or once err < threshold, and
 *     prints "Total steps: %ld; error: %10.6e" (:267);
 *   - without a file argument it prints "Usage:\nppf filename" and exits
 *     with -1 (:122-125).
 * Defaults are the reference's compile-time constants (:15, :92, :99,
 * :104-105); options make them run-time:
 *   --bc periodic|noflux   boundary condition        (default noflux, :15)
 *   --steps N              n_iter                    (default 5000001)
 *   --save N               n_save                    (default 50000)
 *   --init N               n_iter_init               (default 100000000)
 *   --dt X                 time step                 (default 0.125 dx^2/DL)
 *   --threshold X          convergence threshold     (default 1e-12)
 *   --precision f64|f32    device precision          (default f64)
 *   --chunk CZ CY CX       write chunked datasets (the MPI build's layout,
 *                          :574-582) instead of contiguous ones
 *   --ref-etaL-bug         behave like the unmodified reference, whose
 *                          /etaL read goes through the closed /etaS
 *                          identifier (:1032) and leaves etaL = 1.0
 *   --timing               print step throughput on stderr at the end
 *   --mass-project         FP32 runs: put sum(c) back on its initial value
 *                          (FP64 arithmetic, ppf_mass_project) before every
 *                          save, so the solute mass does not drift with the
 *                          FP32 rounding of the per-cell update
 *   --restart              continue the run a saved file belongs to: every
 *                          file written holds a dataset /ppf_restart =
 *                          (next iteration, dt, save number, error); with
 *                          --restart the loop resumes there (same save
 *                          iterations, numbering continued from that save,
 *                          same convergence test, dt from the file unless
 *                          --dt is given), so a restarted run writes what
 *                          the uninterrupted run would have written
 */
#define _POSIX_C_SOURCE 200809L
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "ppf.h"
#include "ppf_h5.h"

#define STD_BUF stderr

static double now_s(void)
{
    struct timespec t;
    clock_gettime(CLOCK_MONOTONIC, &t);
    return (double)t.tv_sec + 1e-9 * (double)t.tv_nsec;
}

static int die(const char *what, const char *msg)
{
    fprintf(stderr, "ppf: %s: %s\n", what, msg);
    return 1;
}

/* smallest save iteration >= i (i > 0 required by :221) */
static int64_t next_save(int64_t i, int64_t n_save, int64_t n_iter_init)
{
    int64_t s = i < 1 ? 1 : i;
    int64_t a = ((s + n_save - 1) / n_save) * n_save;
    if (n_iter_init >= s && n_iter_init < a) a = n_iter_init;
    return a;
}

int main(int argc, char **argv)
{
    if (argc < 2 || argv[1][0] == '-') {
        fprintf(STD_BUF, "Usage:\nppf filename\n");
        return -1;
    }
    const char *input = argv[1];
    int bc = PPF_BC_NOFLUX, prec = PPF_F64, etaL_bug = 0, timing = 0, restart = 0, dt_given = 0, mproj = 0;
    int64_t n_iter = 5000001L, n_save = 50000L, n_iter_init = 100000000L;
    double threshold = 1.0e-12, dt = 0.0;
    int64_t chunk[3] = {0, 0, 0};
    for (int a = 2; a < argc; ++a) {
        const char *o = argv[a];
        int more = a + 1 < argc;
        if (!strcmp(o, "--bc") && more) {
            const char *v = argv[++a];
            if (!strcmp(v, "periodic") || !strcmp(v, "0")) bc = PPF_BC_PERIODIC;
            else if (!strcmp(v, "noflux") || !strcmp(v, "1")) bc = PPF_BC_NOFLUX;
            else return die("--bc", "expected periodic or noflux");
        } else if (!strcmp(o, "--steps") && more) n_iter = strtoll(argv[++a], NULL, 10);
        else if (!strcmp(o, "--save") && more) n_save = strtoll(argv[++a], NULL, 10);
        else if (!strcmp(o, "--init") && more) n_iter_init = strtoll(argv[++a], NULL, 10);
        else if (!strcmp(o, "--dt") && more) { dt = strtod(argv[++a], NULL); dt_given = 1; }
        else if (!strcmp(o, "--threshold") && more) threshold = strtod(argv[++a], NULL);
        else if (!strcmp(o, "--precision") && more) {
            const char *v = argv[++a];
            if (!strcmp(v, "f64")) prec = PPF_F64;
            else if (!strcmp(v, "f32")) prec = PPF_F32;
            else return die("--precision", "expected f64 or f32");
        } else if (!strcmp(o, "--chunk") && a + 3 < argc) {
            for (int q = 0; q < 3; ++q) chunk[q] = strtoll(argv[++a], NULL, 10);
        } else if (!strcmp(o, "--ref-etaL-bug")) etaL_bug = 1;
        else if (!strcmp(o, "--timing")) timing = 1;
        else if (!strcmp(o, "--restart")) restart = 1;
        else if (!strcmp(o, "--mass-project")) mproj = 1;
        else {
            fprintf(STD_BUF, "Usage:\nppf filename\n");
            return -1;
        }
    }
    if (n_save < 1 || n_iter < 0) return die("options", "--save must be >= 1 and --steps >= 0");

    /* job name, phasefield.c:117-121 (without the 50-byte buffer) */
    size_t len = strlen(input);
    if (len < 3) return die(input, "file name too short");
    char *jobname = (char *)malloc(len + 1);
    memcpy(jobname, input, len + 1);
    jobname[len - 3] = '_';
    jobname[len - 2] = '\0';
    fprintf(STD_BUF, "The job name is %s\n", jobname);

    /* read the input, :171-173 */
    int64_t dims[3], d2[3];
    if (ppf_h5_dims(input, "/etaS", dims) != 0) return die(input, ppf_h5_last_error());
    const int64_t n = dims[0] * dims[1] * dims[2];
    double *etaS = (double *)malloc((size_t)n * sizeof(double));
    double *etaL = (double *)malloc((size_t)n * sizeof(double));
    double *c = (double *)malloc((size_t)n * sizeof(double));
    if (!etaS || !etaL || !c) return die("host", "out of memory");
    if (ppf_h5_read3d(input, "/etaS", d2, etaS, n) != 0) return die(input, ppf_h5_last_error());
    if (etaL_bug) {
        for (int64_t q = 0; q < n; ++q) etaL[q] = 1.0;     /* the init value, :160 */
    } else {
        if (ppf_h5_read3d(input, "/etaL", d2, etaL, n) != 0) return die(input, ppf_h5_last_error());
        if (memcmp(d2, dims, sizeof dims)) return die(input, "/etaL and /etaS differ in size");
    }
    if (ppf_h5_read3d(input, "/c", d2, c, n) != 0) return die(input, ppf_h5_last_error());
    if (memcmp(d2, dims, sizeof dims)) return die(input, "/c and /etaS differ in size");

    /* restart record written with every save (see --restart) */
    int64_t i_start = 0;
    int save_start = 0;
    double error_start = threshold;
    if (restart) {
        int64_t rd[3];
        double rec[4];
        if (ppf_h5_dims(input, "/ppf_restart", rd) != 0) return die(input, "no /ppf_restart record to restart from");
        if (rd[0] != 1 || rd[1] != 1 || rd[2] != 4 || ppf_h5_read3d(input, "/ppf_restart", rd, rec, 4) != 0)
            return die(input, "malformed /ppf_restart record");
        if (!(rec[0] >= 0) || !(rec[1] > 0) || !(rec[2] >= 0)) return die(input, "malformed /ppf_restart record");
        i_start = (int64_t)rec[0];
        save_start = (int)rec[2];
        error_start = rec[3];
        if (!dt_given) dt = rec[1];
    }

    ppf_params prm;
    ppf_params_default(&prm);
    prm.dt = dt;
    ppf_derived der;
    if (ppf_params_derive(&prm, &der) != 0) return die("parameters", ppf_last_error());
    ppf_ctx *ctx = NULL;
    if (ppf_create((int)dims[0], (int)dims[1], (int)dims[2], &prm, bc, prec, &ctx) != 0)
        return die("device", ppf_last_error());
    if (ppf_upload(ctx, etaS, etaL, c) != 0) return die("upload", ppf_last_error());
    if (mproj && prec != PPF_F32) return die("--mass-project", "applies to --precision f32");
    double mass0 = 0.0;
    if (mproj) {
        ppf_stats st0;
        if (ppf_reduce(ctx, &st0) != 0) return die("reduce", ppf_last_error());
        mass0 = st0.mass;
    }

    /* main loop, :178-258 */
    int64_t i_iter = i_start;
    double error = error_start;
    int save_iter = save_start;
    double t_steps = 0.0;
    int64_t n_steps = 0;
    char *fname = (char *)malloc(len + 32);
    while (i_iter < n_iter && error >= threshold) {
        int64_t j = next_save(i_iter, n_save, n_iter_init);
        int64_t end = j < n_iter ? j + 1 : n_iter;
        double t0 = now_s();
        int64_t full_end = end < n_iter_init ? end : (i_iter > n_iter_init ? i_iter : n_iter_init);
        if (full_end > i_iter && ppf_step(ctx, full_end - i_iter) != 0) return die("step", ppf_last_error());
        if (end > full_end && ppf_step_c_only(ctx, end - full_end) != 0) return die("step", ppf_last_error());
        if (ppf_sync(ctx) != 0) return die("step", ppf_last_error());
        t_steps += now_s() - t0;
        n_steps += end - i_iter;
        i_iter = end;
        if (j >= n_iter) break;
        /* save step j, :221-256 */
        save_iter++;
        ppf_stats st;
        if (ppf_reduce(ctx, &st) != 0) return die("reduce", ppf_last_error());
        if (mproj && ppf_mass_project(ctx, mass0) != 0) return die("mass projection", ppf_last_error());
        fprintf(STD_BUF, "%ld: c=%10.4e; S=%10.4e; L=%10.4e\t", (long)j, st.sum_dc2, st.sum_detaS2, st.sum_detaL2);
        error = sqrt(st.sum_dc2);
        fprintf(STD_BUF, "iter: %ld; err: %10.4e\n", (long)j, error);
        snprintf(fname, len + 32, "%s%d.h5", jobname, save_iter);
        printf("%s\n", fname);
        fflush(stdout);
        if (ppf_download(ctx, etaS, etaL, c) != 0) return die("download", ppf_last_error());
        const char *names[3] = {"etaS", "etaL", "c"};
        const double *data[3] = {etaS, etaL, c};
        const double rec[4] = {(double)i_iter, der.dt, (double)save_iter, error};
        if (ppf_h5_write3d_meta(fname, 3, names, data, dims, PPF_H5_F64, chunk[0] > 0 ? chunk : NULL, "ppf_restart",
                                rec, 4) != 0)
            return die(fname, ppf_h5_last_error());
    }
    if (timing && t_steps > 0)
        fprintf(STD_BUF, "ppf: %ld steps of %ldx%ldx%ld in %.6f s: %.3f GLUPS\n", (long)n_steps, (long)dims[0],
                (long)dims[1], (long)dims[2], t_steps, (double)n * (double)n_steps / t_steps * 1e-9);
    fprintf(STD_BUF, "Total steps: %ld; error: %10.6e\n", (long)i_iter, error);
    ppf_destroy(ctx);
    free(etaS); free(etaL); free(c); free(fname); free(jobname);
    return 0;
}
