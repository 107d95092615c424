/*
 * cli_gpu_hybrid.cpp -- `gpu_hybrid`, the reference's hybrid solver command
 * line (gpu/hybrid.cu:631-836) over libpcagb.so.
 *
 *   gpu_hybrid <task.json> <max_kernel_depth> [max_solutions=32]
 *              [split_depth=auto] [batch_size=4096]
 *
 * Same positional arguments, the same report lines ("=== depth D (split:
 * CPU s + GPU g) ===", "Optimal solution length: N instructions (kernel
 * depth K)", one "Solution #i  len=L  cpu_verify=p/t OK" block per program,
 * "Total elapsed") and the same exit code (0 iff found). The split depth is
 * the deepest level built on the device with the exact pruner (the
 * reference's CPU prefix DFS runs on the GPU here); batch_size is accepted
 * and unused, since prefixes never cross the bus. Branchless search only.
 */
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "../../include/pca_gb300.h"

int main(int argc, char **argv)
{
    if (argc < 3) {
        fprintf(stderr, "Usage: gpu_hybrid <task.json> <max_kernel_depth> "
                        "[max_solutions] [split_depth] [batch_size]\n");
        return 1;
    }
    const int max_depth = atoi(argv[2]);
    const int max_solutions = argc >= 4 ? atoi(argv[3]) : 32;
    const int user_split = argc >= 5 ? atoi(argv[4]) : -1;
    task_spec_t spec;
    if (task_load(argv[1], &spec) < 0) return 1;
    if (spec.num_outputs != 1) { fprintf(stderr, "multi-output tasks not supported\n"); return 1; }
    if (spec.num_inputs > PCA_NUM_REGS - 1) { fprintf(stderr, "too many inputs\n"); return 1; }
    if (spec.num_inputs + max_depth + 2 > 16) { fprintf(stderr, "program too long\n"); return 1; }
    pcagb_engine_t *e = nullptr;
    if (pcagb_engine_create(0, 0, &e) != PCAGB_OK) {
        fprintf(stderr, "gpu_hybrid: %s\n", pcagb_last_error());
        return 1;
    }
    printf("PCA-16 hybrid CPU-GPU solver\n");
    printf("  task: %s (%s)\n", argv[1], spec.name);
    printf("  tests: %d  inputs: %d  outputs: %d\n", spec.num_tests, spec.num_inputs,
           spec.num_outputs);
    printf("  gpu candidates: %d (root live mask)  branchless\n",
           pcagb_num_candidates((uint8_t)(((1u << spec.num_inputs) - 1u) << 1)));
    auto t0 = std::chrono::steady_clock::now();
    pcagb_opts_t o;
    pcagb_default_opts(&o);
    o.max_depth = max_depth;
    o.split_depth = user_split;
    o.oep_mode = PCAGB_OEP_EXACT_LIVE;
    const int cap = max_solutions > 0 ? max_solutions : 1;
    std::vector<uint16_t> progs((size_t)cap * 16);
    std::vector<int> lens(cap);
    pcagb_result_t r;
    int rc = pcagb_solve(e, &spec, &o, &r, progs.data(), lens.data(), cap);
    double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (rc != PCAGB_OK) {
        fprintf(stderr, "gpu_hybrid: %s\n", pcagb_last_error());
        pcagb_engine_destroy(e);
        return 1;
    }
    const int last = r.optimal_depth >= 0 ? r.optimal_depth : max_depth;
    for (int k = 0; k <= last; k++) {
        int split = user_split >= 0 ? (user_split < k ? user_split : k) : (k > 0 ? k - 1 : 0);
        if (k == last) split = r.split_used < k ? r.split_used : split;
        printf("\n=== depth %d (split: CPU %d + GPU %d) ===\n", k, split, k - split);
        printf("  gpu: %llu candidates decided, %llu value-class evaluations\n",
               (unsigned long long)r.candidates[k], (unsigned long long)r.evaluations[k]);
        if (k < last || r.optimal_depth < 0) printf("  solutions: 0\n");
    }
    if (r.optimal_depth >= 0) {
        printf("\nOptimal solution length: %d instructions (kernel depth %d)\n",
               spec.num_inputs + r.optimal_depth + 2, r.optimal_depth);
        char buf[64];
        for (int i = 0; i < r.stored; i++) {
            const uint16_t *p = &progs[(size_t)i * 16];
            int passed = task_evaluate(&spec, p, lens[i]);
            printf("\nSolution #%d  len=%d  cpu_verify=%d/%d %s\n", i + 1, lens[i], passed,
                   spec.num_tests, passed == spec.num_tests ? "OK" : "FAIL");
            for (int j = 0; j < lens[i]; j++) {
                pca_disasm(p[j], buf, sizeof buf);
                printf("    %02X: %04X  %s\n", j, p[j], buf);
            }
        }
    }
    printf("\nTotal elapsed: %.3f sec\n", secs);
    pcagb_engine_destroy(e);
    return r.optimal_depth >= 0 ? 0 : 1;
}
