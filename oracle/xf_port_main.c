/*
 * Oracle (test infrastructure only).  Command-line driver for the C
 * restatement: runs the evolution loop (src/Nmr.cpp:89-262) on a config for a
 * bounded number of iterations and prints one JSON line with the loop's wall
 * time, in the manner of the reference's own DBG "total time" line
 * (src/Nmr.cpp:253-255).  Used to time the CPU baseline.
 *
 * usage: xfport <config> [--iters N] [--r0 R] [--dr DR] [--noise SEED AMP]
 */
#define _POSIX_C_SOURCE 200809L
#include "xf_port.h"
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#ifdef _OPENMP
#include <omp.h>
#endif

int main(int argc, char** argv)
{
    if (argc < 2) { fprintf(stderr, "usage: %s <config> [--iters N] [--r0 R] [--dr DR] [--noise SEED AMP]\n", argv[0]); return 2; }
    xfp_sim* s = xfp_create(argv[1]);
    if (!s) { fprintf(stderr, "cannot load config %s\n", argv[1]); return 2; }
    double prm[10];
    xfp_params(s, prm);
    double r0 = prm[0], dr0 = prm[2];
    long iters = -1;
    unsigned long long seed = (unsigned long long)prm[8];
    double amp = prm[9];
    for (int i = 2; i < argc; ++i) {
        if (!strcmp(argv[i], "--iters") && i + 1 < argc) iters = atol(argv[++i]);
        else if (!strcmp(argv[i], "--r0") && i + 1 < argc) r0 = atof(argv[++i]);
        else if (!strcmp(argv[i], "--dr") && i + 1 < argc) dr0 = atof(argv[++i]);
        else if (!strcmp(argv[i], "--noise") && i + 2 < argc) { seed = strtoull(argv[i + 1], 0, 10); amp = atof(argv[i + 2]); i += 2; }
        else { fprintf(stderr, "unknown option %s\n", argv[i]); return 2; }
    }
    if (amp > 0) xfp_noise(s, seed, amp);
    struct timespec t0, t1;
    clock_gettime(CLOCK_MONOTONIC, &t0);
    long n_acc = 0;
    double r_end = 0, dr_end = 0;
    long it = xfp_run(s, r0, dr0, iters, NULL, 0, &n_acc, &r_end, &dr_end);
    clock_gettime(CLOCK_MONOTONIC, &t1);
    double secs = (t1.tv_sec - t0.tv_sec) + 1e-9 * (t1.tv_nsec - t0.tv_nsec);
    int threads = 1;
#ifdef _OPENMP
    threads = omp_get_max_threads();
#endif
    double bins = (double)xfp_nbeams(s) * xfp_ebins(s);
    printf("{\"iterations\": %ld, \"accepted\": %ld, \"seconds\": %.6f, \"bins\": %.0f, \"threads\": %d, "
           "\"r_end\": %.17g, \"dr_end\": %.17g, \"bin_iter_per_s\": %.6e}\n",
           it, n_acc, secs, bins, threads, r_end, dr_end, bins * it / secs);
    xfp_destroy(s);
    return 0;
}
