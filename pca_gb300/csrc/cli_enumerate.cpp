/*
 * cli_enumerate.cpp -- `enumerate`, the reference solver's command line
 * (tools/enumerate.c:537-755) over libpcagb.so.
 *
 *   enumerate <task.json> [-d max_depth] [--no-branch] [--no-oep] [-v] [--count]
 *   enumerate <task.json> [-d max_depth] --no-branch --record <output_dir>
 *             [--task-id N] [--neg-stride N]
 *
 * Same argument grammar, the same report lines (task summary, per-depth
 * "candidates" / "OEP pruned" / "solutions found" / "elapsed", the solutions
 * with their disassembly and test[0] check, "Optimal solution length: N
 * instructions (kernel depth K)", "Found N distinct program(s) at this
 * length.") and the same exit code (0 iff a program was found).
 *
 * The search runs on the GPU. Without --no-branch it is the reference's
 * branch mode (CMP, forward BR, DIV, MOD; pcagb_solve_branch) with its
 * per-depth counters; with --no-branch the branchless engine. With OEP on,
 * the pruner is exact (key regs+flags, DFS-first representative,
 * full-state compare); the printed programs are the reference's (its
 * DFS-first program per final state, at most 100). --count builds every level with the pruner so the per-depth
 * counters are the reference's exact-pruner counters; without it the search
 * builds levels only as deep as HBM allows and enumerates the rest, and the
 * counters are this engine's.
 *
 * --record writes the reference's training records (tools/enumerate.c:
 * 676-740) from the GPU levels through pcagb_record: states_<id>.bin and
 * edges_<id>.bin with the same records in the same order, and the same
 * report lines; as in the reference, the closing "Total" line then counts
 * the recording pass (the optimal depth's search) alone.
 */
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "../../include/pca_gb300.h"

static void print_solution(const task_spec_t &t, const uint16_t *p, int len, int idx)
{
    printf("  Solution #%d (%d instructions):\n", idx + 1, len);
    char buf[64];
    for (int i = 0; i < len; i++) {
        pca_disasm(p[i], buf, sizeof buf);
        printf("    %02X: %04X  %s\n", i, p[i], buf);
    }
    pca_vm_t vm;
    pca_init(&vm);
    pca_load(&vm, p, (size_t)len);
    for (int i = 0; i < t.num_inputs; i++) vm.ports[t.input_ports[i]] = t.tests[0].in[i];
    pca_run(&vm, t.max_cycles);
    printf("    verify test[0]: in=(");
    for (int i = 0; i < t.num_inputs; i++) printf("%s%u", i ? "," : "", t.tests[0].in[i]);
    uint16_t got = vm.ports[t.output_ports[0]];
    printf(") -> port%d=%u (expected %u) %s\n", t.output_ports[0], got, t.tests[0].out[0],
           got == t.tests[0].out[0] ? "OK" : "FAIL");
}

int main(int argc, char **argv)
{
    if (argc < 2) {
        fprintf(stderr,
                "Usage: enumerate <task.json> [-d max_depth] [--no-branch] [--no-oep] [-v] [--count]\n"
                "       enumerate <task.json> [-d max_depth] --record <output_dir> "
                "[--task-id N] [--neg-stride N]\n");
        return 1;
    }
    int max_depth = 4, no_branch = 0, no_oep = 0, count = 0, neg_stride = 8;
    const char *record_dir = nullptr;
    uint32_t task_id = 0;
    for (int i = 2; i < argc; i++) {
        if (!strcmp(argv[i], "-d") && i + 1 < argc) max_depth = atoi(argv[++i]);
        else if (!strcmp(argv[i], "--no-branch")) no_branch = 1;
        else if (!strcmp(argv[i], "--no-oep")) no_oep = 1;
        else if (!strcmp(argv[i], "--count")) count = 1;
        else if (!strcmp(argv[i], "-v")) {
        } else if (!strcmp(argv[i], "--record") && i + 1 < argc) record_dir = argv[++i];
        else if (!strcmp(argv[i], "--task-id") && i + 1 < argc) task_id = (uint32_t)atoi(argv[++i]);
        else if (!strcmp(argv[i], "--neg-stride") && i + 1 < argc) neg_stride = atoi(argv[++i]);
    }
    /* recording is branchless and builds every level with the pruner */
    if (record_dir) {
        if (no_oep) {
            fprintf(stderr, "enumerate: --record without the pruner (--no-oep) is not supported\n");
            return 2;
        }
        no_branch = 1;
        count = 1;
    }
    task_spec_t task;
    if (task_load(argv[1], &task) < 0) return 1;
    task_print(&task);
    printf("\n");
    if (!no_branch && no_oep) {
        fprintf(stderr, "enumerate: branch mode without the pruner (--no-oep) is not supported\n");
        return 2;
    }
    pcagb_engine_t *e = nullptr;
    /* branch mode keeps its levels outside the engine's arena */
    if (pcagb_engine_create(0, no_branch ? 0 : ((size_t)1 << 30), &e) != PCAGB_OK) {
        fprintf(stderr, "enumerate: %s\n", pcagb_last_error());
        return 1;
    }
    if (!no_branch) {
        printf("Enumerating programs (max kernel depth %d, branches on, OEP on)...\n\n", max_depth);
        const int bcap = 100;
        std::vector<uint16_t> bprogs(bcap * 16);
        std::vector<int> blens(bcap);
        pcagb_result_t br;
        auto b0 = std::chrono::steady_clock::now();
        int brc = pcagb_solve_branch(e, &task, max_depth, &br, bprogs.data(), blens.data(), bcap);
        double bsecs = std::chrono::duration<double>(std::chrono::steady_clock::now() - b0).count();
        if (brc != PCAGB_OK) {
            fprintf(stderr, "enumerate: %s\n", pcagb_branch_last_error());
            pcagb_engine_destroy(e);
            return 1;
        }
        const int blast = br.optimal_depth >= 0 ? br.optimal_depth : max_depth;
        uint64_t btotal = 0;
        for (int k = 0; k <= blast; k++) {
            printf("--- kernel depth %d (total program length %d) ---\n", k, task.num_inputs + k + 2);
            btotal += br.tried[k];
            const int found = k == br.optimal_depth ? (int)br.total_solutions : 0;
            printf("  candidates: %llu  (%.1f M/sec)\n", (unsigned long long)br.tried[k],
                   bsecs > 0 ? br.tried[k] / bsecs / 1e6 : 0.0);
            printf("  OEP pruned: %llu\n", (unsigned long long)br.pruned_cum[k]);
            printf("  solutions found: %d (total: %d)\n", found, found);
            printf("  elapsed: %.2f sec\n\n", bsecs);
            if (found)
                for (int i = 0; i < br.stored; i++) print_solution(task, &bprogs[i * 16], blens[i], i);
        }
        if (br.optimal_depth < 0) {
            printf("\nNo solutions found up to kernel depth %d.\n", max_depth);
            pcagb_engine_destroy(e);
            return 1;
        }
        printf("\nOptimal solution length: %d instructions (kernel depth %d)\n",
               task.num_inputs + br.optimal_depth + 2, br.optimal_depth);
        printf("Found %d distinct program(s) at this length.\n", (int)br.total_solutions);
        printf("\nTotal: %llu candidates in %.2f sec (OEP pruned: %llu)\n", (unsigned long long)btotal,
               bsecs, (unsigned long long)br.pruned_cum[blast]);
        pcagb_engine_destroy(e);
        return 0;
    }
    printf("Enumerating programs (max kernel depth %d, branches off, OEP %s, search_state)...\n\n",
           max_depth, no_oep ? "off" : "on");
    pcagb_opts_t o;
    pcagb_default_opts(&o);
    o.max_depth = max_depth;
    o.oep_mode = no_oep ? PCAGB_OEP_NONE : PCAGB_OEP_EXACT;
    o.count_levels = count || no_oep;
    const int cap = 100;
    std::vector<uint16_t> progs(cap * 16);
    std::vector<int> lens(cap);
    pcagb_result_t r;
    auto t0 = std::chrono::steady_clock::now();
    int rc = pcagb_solve(e, &task, &o, &r, progs.data(), lens.data(), cap);
    double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (rc != PCAGB_OK) {
        fprintf(stderr, "enumerate: %s\n", pcagb_last_error());
        pcagb_engine_destroy(e);
        return 1;
    }
    const int last = r.optimal_depth >= 0 ? r.optimal_depth : max_depth;
    uint64_t total_tried = 0;
    for (int k = 0; k <= last; k++) {
        printf("--- kernel depth %d (total program length %d) ---\n", k, task.num_inputs + k + 2);
        total_tried += r.tried[k];
        const int found = k == r.optimal_depth ? r.stored : 0;
        printf("  candidates: %llu  (%.1f M/sec)\n", (unsigned long long)r.tried[k],
               secs > 0 ? r.tried[k] / secs / 1e6 : 0.0);
        if (!no_oep) printf("  OEP pruned: %llu\n", (unsigned long long)r.pruned_cum[k]);
        printf("  solutions found: %d (total: %d)\n", found, found);
        printf("  elapsed: %.2f sec\n\n", secs);
        if (found)
            for (int i = 0; i < r.stored; i++) print_solution(task, &progs[i * 16], lens[i], i);
    }
    if (r.optimal_depth < 0) {
        printf("\nNo solutions found up to kernel depth %d.\n", max_depth);
        pcagb_engine_destroy(e);
        return 1;
    }
    printf("\nOptimal solution length: %d instructions (kernel depth %d)\n",
           task.num_inputs + r.optimal_depth + 2, r.optimal_depth);
    printf("Found %d distinct program(s) at this length.\n", r.stored);
    uint64_t pruned_total = r.pruned_cum[last];
    if (record_dir) {
        const int K = r.optimal_depth;
        printf("\n===== Recording dataset (Pass 2) =====\n");
        printf("  building optimal state sets from %d solutions...\n", r.stored);
        auto r0 = std::chrono::steady_clock::now();
        pcagb_record_stats_t st;
        int rrc = pcagb_record(e, &task, max_depth, task_id, neg_stride, record_dir, &st);
        double rsecs = std::chrono::duration<double>(std::chrono::steady_clock::now() - r0).count();
        if (rrc < 0) {
            fprintf(stderr, "enumerate: %s\n", pcagb_last_error());
            pcagb_engine_destroy(e);
            return 1;
        }
        printf("  optimal state set: %d states across %d depths\n", st.optimal_states, K + 1);
        printf("  recording done in %.2f sec\n", rsecs);
        printf("  states: %llu written (%llu positive, %llu negative)\n",
               (unsigned long long)st.states_written, (unsigned long long)st.positives,
               (unsigned long long)st.negatives);
        printf("  edges: %llu written\n", (unsigned long long)st.edges_written);
        /* the reference resets its counters for the recording pass */
        total_tried = r.tried[K];
        pruned_total = r.pruned_cum[K] - (K > 0 ? r.pruned_cum[K - 1] : 0);
    }
    printf("\nTotal: %llu candidates in %.2f sec", (unsigned long long)total_tried, secs);
    if (!no_oep) printf(" (OEP pruned: %llu)", (unsigned long long)pruned_total);
    printf("\n");
    pcagb_engine_destroy(e);
    return 0;
}
