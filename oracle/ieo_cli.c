/* ieo_cli.c -- command-line runner of the CPU oracle (test infrastructure).
 * Usage: ieo_cli <params.txt> <results_dir> <inputs_dir> [threads] */
#include "ieo.h"
#include <stdio.h>
#include <stdlib.h>

int main(int argc, char** argv) {
    if (argc < 4) {
        fprintf(stderr, "usage: ieo_cli <params.txt> <results_dir> <inputs_dir> [threads]\n");
        return 2;
    }
    ieo_params p;
    ieo_params_defaults(&p, 16, 0);
    /* first pass: N and potential kind decide the defaults */
    ieo_params q = p;
    ieo_params_load(&q, argv[1]);
    ieo_params_defaults(&p, q.N, q.numerical_potential);
    p.perform_deltaN = q.perform_deltaN;
    p.calculate_SIGW = q.calculate_SIGW;
    ieo_params_load(&p, argv[1]);
    if (argc > 4) ieo_set_threads(atoi(argv[4]));
    return ieo_run_program(&p, argv[2], argv[3]);
}
