/*
 * oracle_cli.c -- command-line front end of the CPU oracle (test
 * infrastructure). Prints the per-depth counters of tools/enumerate.c:624-662
 * so its output can be compared line by line with the reference solver.
 *
 *   oracle_enumerate <task.json> [-d D] [--mode ref32|exact|exact-live|none]
 *                    [--all]
 */
#include "pca_oracle.h"
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

int main(int argc, char **argv)
{
    if (argc < 2) {
        fprintf(stderr, "usage: oracle_enumerate <task.json> [-d D] [--mode M] [--all]\n");
        return 2;
    }
    int depth = 4, mode = ORC_OEP_REF32, cap = -1;
    for (int i = 2; i < argc; i++) {
        if (!strcmp(argv[i], "-d") && i + 1 < argc) depth = atoi(argv[++i]);
        else if (!strcmp(argv[i], "--all")) cap = 1 << 16;
        else if (!strcmp(argv[i], "--mode") && i + 1 < argc) {
            const char *m = argv[++i];
            mode = !strcmp(m, "none") ? ORC_OEP_NONE : !strcmp(m, "exact") ? ORC_OEP_EXACT
                 : !strcmp(m, "exact-live") ? ORC_OEP_EXACT_LIVE : ORC_OEP_REF32;
        }
    }
    orc_task_t task;
    if (orc_task_load(argv[1], &task) < 0) return 1;
    int n = cap < 0 ? 100 : cap;
    uint16_t *progs = calloc((size_t)n * 16, 2);
    int *lens = calloc((size_t)n, sizeof(int));
    orc_result_t r;
    if (orc_enumerate(&task, depth, mode, cap, progs, lens, &r) < 0) return 1;
    int last = r.optimal_depth >= 0 ? r.optimal_depth : depth;
    for (int k = 0; k <= last; k++)
        printf("depth %d candidates %llu pruned %llu solutions %d\n", k,
               (unsigned long long)r.tried[k], (unsigned long long)r.pruned_cum[k], r.sols_at[k]);
    for (int k = 0; k <= last; k++)
        printf("level %d children %llu survivors %llu\n", k,
               (unsigned long long)r.children[k], (unsigned long long)r.survivors[k]);
    if (r.optimal_depth < 0) {
        printf("No solutions found up to kernel depth %d.\n", depth);
        return 1;
    }
    printf("Optimal solution length: %d instructions (kernel depth %d)\n",
           task.num_inputs + r.optimal_depth + 2, r.optimal_depth);
    printf("Found %llu distinct program(s) at this length.\n", (unsigned long long)r.total_solutions);
    for (int i = 0; i < r.num_solutions; i++) {
        printf("sol");
        for (int j = 0; j < lens[i]; j++) printf(" %04X", progs[i * 16 + j]);
        printf("\n");
    }
    return 0;
}
