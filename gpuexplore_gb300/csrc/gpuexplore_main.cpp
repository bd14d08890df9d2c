// gpuexplore_main.cpp -- the `gpuexplore` command-line tool, a client of libgpx.
//
// Same invocation, flag semantics and result lines as the reference's main
// (GPUexplore.cu:1738-2188):
//   gpuexplore <model> [-b N] [-t N] [-k N] [-q N] [-v N] [--por] [--cycle-proviso]
//              [-d|-p] [--dump FILE] [-h]
// plus this build's additions: --seed N, --max-states N, --store N, --device N.
#include <chrono>
#include <cinttypes>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

#include "gpx.h"

static const char *kHelp =
    "Usage: gpuexplore <model> [OPTIONS]\n"
    "Run state-space exploration on model (do not include the file extension).\n"
    "options:\n"
    "  -d                 Check for deadlocks\n"
    "  -p                 Check a safety property (should be embedded in the model)\n"
    "  --por              Apply partial-order reduction\n"
    "  --cycle-proviso    Apply the cycle proviso during partial-order reduction\n"
    "  -k NUM             Run NUM BFS levels per kernel launch (default 0: one launch to the end)\n"
    "  -b NUM             Run the kernel on NUM blocks (default: every SM at full occupancy)\n"
    "  -t NUM             Use NUM threads per block (default 256, at most 256)\n"
    "  -q NUM             Allocate NUM integers for the hash table\n"
    "  --dump FILE        Dump the state space to FILE after completing the exploration\n"
    "  -v NUM             Change the verbosity:\n"
    "                        0 - minimal output\n"
    "                        1 - print sequence number of each kernel launch\n"
    "                        2 - print number of states in the hash table after each kernel launch\n"
    "                        3 - print state vectors after each kernel launch\n"
    "  --seed NUM         Seed of the hash functions\n"
    "  --max-states NUM   Stop at the end of the BFS level that reaches NUM states\n"
    "  --store NUM        Capacity of the state store in states\n"
    "  --device NUM       CUDA device to use\n"
    "  --por-model FILE   Use the learned cluster proposal in FILE (a gpx_por_model) with --por\n"
    "  --ample            Partial-order reduction with single-process ample sets\n"
    "  --stubborn         Partial-order reduction with stubborn sets (necessary enabling processes)\n"
    "  --no-prune         Generate every successor in plain exploration (no commuting-move pruning)\n"
    "  -h, --help         Show this help message\n";

static uint64_t mix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

int main(int argc, char **argv) {
    auto start = std::chrono::steady_clock::now();
    if (argc == 1) {
        fprintf(stderr, "ERROR: No input network given!\n");
        fputs(kHelp, stdout);
        return 1;
    }
    if (!strcmp(argv[1], "--help") || !strcmp(argv[1], "-h") || !strcmp(argv[1], "-?")) {
        fputs(kHelp, stdout);
        return 0;
    }
    gpx_options o;
    gpx_options_init(&o);
    const char *dump_file = nullptr;
    const char *por_model_file = nullptr;
    int i = 2;
    auto need = [&](int k) {
        if (k + 1 >= argc) {
            fprintf(stderr, "ERROR: option %s needs a value\n", argv[k]);
            fputs(kHelp, stdout);
            exit(1);
        }
        return argv[k + 1];
    };
    // option semantics of GPUexplore.cu:1817-1883
    while (i < argc) {
        const char *a = argv[i];
        if (!strcmp(a, "--help") || !strcmp(a, "-h") || !strcmp(a, "-?")) {
            fputs(kHelp, stdout);
            return 0;
        } else if (!strcmp(a, "-k")) {
            o.kernel_iters = atoi(need(i));
            i += 2;
        } else if (!strcmp(a, "-b")) {
            o.blocks = atoi(need(i));
            i += 2;
        } else if (!strcmp(a, "-t")) {
            o.threads = atoi(need(i));
            i += 2;
        } else if (!strcmp(a, "-q")) {
            o.q_words = strtoull(need(i), nullptr, 10);
            i += 2;
        } else if (!strcmp(a, "-v")) {
            o.verbosity = atoi(need(i));
            if (o.verbosity > 3) o.verbosity = 3;
            i += 2;
        } else if (!strcmp(a, "-d")) {
            o.property = GPX_PROP_DEADLOCK; // -d switches the cycle proviso off
            o.cycle_proviso = 0;
            i += 1;
        } else if (!strcmp(a, "-p")) {
            o.property = GPX_PROP_SAFETY; // -p switches the cycle proviso on
            o.cycle_proviso = 1;
            i += 1;
        } else if (!strcmp(a, "--por")) {
            if (!o.por) o.por = 1;
            i += 1;
        } else if (!strcmp(a, "--ample")) {
            o.por = 3; // single-process ample sets
            i += 1;
        } else if (!strcmp(a, "--stubborn")) {
            o.por = 4; // stubborn sets from necessary enabling processes
            i += 1;
        } else if (!strcmp(a, "--no-prune")) {
            o.prune_commuting = 0;
            i += 1;
        } else if (!strcmp(a, "--cycle-proviso")) {
            if (o.property == GPX_PROP_NONE) o.cycle_proviso = 1; // only before -d/-p
            i += 1;
        } else if (!strcmp(a, "--dump")) {
            dump_file = need(i);
            i += 2;
        } else if (!strcmp(a, "--seed")) {
            o.seed = strtoull(need(i), nullptr, 10);
            i += 2;
        } else if (!strcmp(a, "--max-states")) {
            o.max_states = strtoull(need(i), nullptr, 10);
            i += 2;
        } else if (!strcmp(a, "--store")) {
            o.store_states = strtoull(need(i), nullptr, 10);
            i += 2;
        } else if (!strcmp(a, "--device")) {
            o.device = atoi(need(i));
            i += 2;
        } else if (!strcmp(a, "--por-model")) {
            por_model_file = need(i);
            i += 2;
        } else {
            fprintf(stderr, "ERROR: unrecognized option %s\n", a);
            fputs(kHelp, stdout);
            return 1;
        }
    }

    gpx_model *m = nullptr;
    int rc = gpx_model_load(argv[1], &m);
    if (rc == GPX_ERR_PARSE) {
        fprintf(stderr, "ERROR: input network does not exist!\n");
        return 1;
    }
    if (rc != GPX_OK) {
        fprintf(stderr, "ERROR: %s\n", gpx_status_string(rc));
        return 1;
    }
    gpx_model_info info;
    gpx_model_info_get(m, &info);
    // header echo (GPUexplore.cu:1888-1953)
    if (o.property == GPX_PROP_SAFETY) {
        printf("Property to check is %sa liveness property\n", info.liveness == 0 ? "not " : "");
        if (info.liveness == 1) o.property = GPX_PROP_LIVENESS;
    }
    printf("nr of procs: %u\n", info.nr_procs);
    printf("nr of bits for transition label: %u\n", info.bits_act);
    printf("min. nr. of proc. states that fit in 32-bit integer: %u\n", info.proc_nrstates);
    printf("number of bits needed for a state vector: %u\n", info.bits_statevector + (o.por ? 1u : 0u));
    for (uint32_t p = 0; p <= info.nr_procs; p++) printf("statevector offset %u: %u\n", p, info.firstbit[p]);
    for (uint32_t p = 0; p < info.nr_procs; p++) printf("bits for states of process LTS %u: %u\n", p, info.bits_state[p]);
    printf("size of offset in process LTSs: %u\n", info.nbits_offset);
    printf("maximum label-bounded branching factor: %u\n", info.max_buf_ints);
    printf("total number of transition entries in network: %u\n", info.nr_trans);

    gpx_device_info dev;
    if (gpx_device_info_get(o.device, &dev) == GPX_ERR_NO_GPU) {
        fprintf(stderr, "ERROR: No CUDA compatible GPU detected!\n");
        return 1;
    }
    printf("global mem: %" PRIu64 "\n", dev.total_global_mem);
    printf("shared mem per block: %d\n", dev.shared_mem_per_block);
    printf("shared mem per SM: %d\n", dev.shared_mem_per_sm);
    printf("max. threads per block: %d\n", dev.max_threads_per_block);
    printf("max. grid size: %d\n", dev.max_grid_size);
    printf("nr. of multiprocessors: %d\n", dev.sm_count);

    gpx_por_model pm;
    if (por_model_file) {
        FILE *pf = fopen(por_model_file, "rb");
        if (!pf || fread(&pm, sizeof pm, 1, pf) != 1) {
            fprintf(stderr, "ERROR: cannot read POR model %s\n", por_model_file);
            return 1;
        }
        fclose(pf);
        if (o.por == 1) o.por = 2; // the proposal ranks cample's clusters
    }
    gpx_explorer *ex = nullptr;
    rc = gpx_explorer_create(m, &o, &ex);
    if (rc != GPX_OK) {
        fprintf(stderr, "ERROR: %s\n", gpx_status_string(rc));
        return 1;
    }
    if (por_model_file) gpx_explorer_set_por_model(ex, &pm);
    // hash constants derived from the seed (the reference draws 16 with rand(), GPUexplore.cu:1990-1993)
    auto explore_start = std::chrono::steady_clock::now();
    gpx_result r;
    rc = gpx_explorer_run(ex, &r);
    printf("global mem queue size: %" PRIu64 ", number of entries: %" PRIu64 "\n",
           r.table_slots * (uint64_t)r.slot_bytes, r.table_slots);
    printf("nr. of blocks: %u, block size: %u, nr of kernel iterations: %d\n", r.blocks, r.threads, o.kernel_iters);
    for (int k = 0; k < 16; k++) printf("hash constant %d: %d\n", k, (int)(mix64(o.seed + k) & 0x7FFFFFFF));
    auto stop = std::chrono::steady_clock::now();
    printf("Run time: %f\n", std::chrono::duration<double>(stop - start).count());
    printf("Exploration time %f\n", (r.setup_ms + r.explore_ms) / 1000.0);
    if (r.verdict == GPX_PROP_DEADLOCK) printf("deadlock detected!\n");
    if (r.verdict == GPX_PROP_SAFETY) printf("safety property violation detected!\n");
    if (r.verdict == GPX_PROP_LIVENESS) printf("liveness property violation detected!\n");
    if (rc == GPX_ERR_TABLE_FULL) fprintf(stderr, "ERROR: problem with hash table\n");
    else if (rc != GPX_OK) fprintf(stderr, "ERROR: %s\n", gpx_status_string(rc));
    printf("nr. of states in hash table: %" PRIu64 "\n", r.states);
    if (dump_file) {
        FILE *f = fopen(dump_file, "w");
        if (f) {
            fclose(f);
            printf("Dumping state space to file...\n");
            gpx_explorer_dump(ex, dump_file);
        } else {
            fprintf(stderr, "Could not open file to dump the state space\n");
        }
    }
    (void)explore_start;
    gpx_result_free(&r);
    gpx_explorer_destroy(ex);
    gpx_model_free(m);
    return 0;
}
