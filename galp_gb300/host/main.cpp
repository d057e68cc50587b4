// main.cpp -- the `galp` command-line front end, a drop-in for the reference's CLI.
//
// Same usage, options, method/policy table and output as label_propagation/src/main.cu:
//   galp [-b n] [-i n] [-g n] [-l n] method policy data [test]
// prints "Data is ready on the host (n, m)", the "----------<proc>----------" banner,
// one line per iteration, and on stderr the tab-separated result row
//   proc  file  niter  buffer_pow  f1  f2  nmi  fm  ari        (main.cu:240-242)
// The update runs on the GPU through the C ABI in include/galp.h.  Cases the
// reference routes to its hybrid, load-imbalanced, multi-GPU or serial paths
// (main.cu:157-166, 186-206) are reported as not provided and exit with status 1.
// Extra options: --frontier (skip unchanged neighbourhoods), --dispatch=fixed|learned.
#include <getopt.h>
#include <libgen.h>

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <string>
#include <vector>

#include "../../include/galp.h"
#include "../../include/galp_host.h"

static void usage(char *prog)
{
    std::cerr << "Usage: " << prog << " [options] method policy data [test]" << std::endl
              << "  method: Specify the method to be used." << std::endl
              << "    0 -- data-parallel primitives" << std::endl
              << "    1 -- lock-free hash tables" << std::endl
              << "  policy: Specify the policy to perform the method." << std::endl
              << "    0 -- GPU in-core" << std::endl
              << "    1 -- Out-of-core without overlap" << std::endl
              << "    2 -- Out-of-core with overlap" << std::endl
              << "    3 -- CPU-GPU hybrid" << std::endl
              << "    4 -- Depending on the method" << std::endl
              << "      method=0: Load-imbalanced" << std::endl
              << "      method=1: Multi-GPU, out-of-core with overlap" << std::endl
              << "    5 -- Multi-GPU in-core (only for method 1)" << std::endl
              << "  data: The graph data file." << std::endl
              << "  test: The ground-truth file. Accuracy is computed if supplied." << std::endl
              << "Options: " << std::endl
              << " -b n: Set buffer sizes to 2^n. The default is 24." << std::endl
              << " -i n: Specify the number of iterations. The default is 10." << std::endl
              << " -g n: Use n GPUs. The default is 1." << std::endl;
    std::exit(1);
}

int main(int argc, char *argv[])
{
    int buffer_pow = 24, niter = 10, ngpus = 1, lfht_policy = 1;
    int frontier = 0, dispatch = 0;
    static option longopts[] = {{"frontier", no_argument, nullptr, 'F'},
                                {"dispatch", required_argument, nullptr, 'D'},
                                {nullptr, 0, nullptr, 0}};
    int ch;
    while ((ch = getopt_long(argc, argv, "b:i:g:l:", longopts, nullptr)) != -1) {
        switch (ch) {
        case 'b': buffer_pow = std::atoi(optarg); break;
        case 'i': niter = std::atoi(optarg); break;
        case 'g': ngpus = std::atoi(optarg); break;
        case 'l': lfht_policy = std::atoi(optarg); break;
        case 'F': frontier = 1; break;
        case 'D': dispatch = std::strcmp(optarg, "learned") == 0; break;
        default: usage(argv[0]);
        }
    }
    argc -= optind;
    if (argc < 3) usage(argv[0]);
    argv += optind;
    const int method = std::atoi(argv[0]);
    const int policy = std::atoi(argv[1]);
    char *graph_file = argv[2];

    galp_host_graph *g = nullptr;
    if (galp_load_graph(graph_file, &g) != 0) {
        std::cerr << "cannot read " << graph_file << std::endl;
        return 1;
    }
    std::cout << "Data is ready on the host (" << g->n << ", " << g->m << ")" << std::endl;

    galp_opts opts;
    galp_default_opts(&opts);
    opts.lfht_policy = lfht_policy;
    opts.frontier = frontier;
    opts.dispatch = dispatch;
    std::string proc_name;
    const std::string lf = "lfht" + std::to_string(lfht_policy);
    bool provided = true;
    switch (method * 5 + policy) {
    case 0: buffer_pow = 0; proc_name = "dpp\tincore"; opts.method = 0; opts.policy = 0; break;
    case 1: proc_name = "dpp\tsync"; opts.method = 0; opts.policy = 1; break;
    case 2: proc_name = "dpp\tasync"; opts.method = 0; opts.policy = 2; break;
    case 3: proc_name = "dpp\thybrid"; provided = false; break;
    case 4: buffer_pow = 0; proc_name = "dpp\tli"; provided = false; break;
    case 5: buffer_pow = 0; proc_name = lf + "\tincore"; opts.method = 1; opts.policy = 0; break;
    case 6: proc_name = lf + "\tsync"; opts.method = 1; opts.policy = 1; break;
    case 7: proc_name = lf + "\tasync"; opts.method = 1; opts.policy = 2; break;
    case 8: proc_name = lf + "\thybrid"; provided = false; break;
    case 9: proc_name = lf + "\tasync multi" + std::to_string(ngpus); provided = false; break;
    case 10: buffer_pow = 0; proc_name = lf + "\tincore multi" + std::to_string(ngpus); provided = false; break;
    default: buffer_pow = 0; proc_name = "serial\t "; provided = false;
    }
    opts.buffer_pow = buffer_pow;
    std::cout << "----------" << proc_name << "----------" << std::endl;
    if (!provided || ngpus != 1) {
        std::cerr << "galp-gb300: " << proc_name
                  << " is not provided (one GPU; in-core and out-of-core policies 0-2 only)" << std::endl;
        galp_host_graph_free(g);
        return 1;
    }

    galp_csr csr{g->neighbors, g->offsets, g->n, g->m};
    galp_ctx *ctx = nullptr;
    int rc = galp_create(&csr, &opts, &ctx);
    if (rc) {
        std::cerr << "galp_create: " << galp_strerror(rc) << std::endl;
        galp_host_graph_free(g);
        return 1;
    }
    galp_stats st;
    rc = galp_run(ctx, niter, &st);
    if (rc) {
        std::cerr << "galp_run: " << galp_strerror(rc) << std::endl;
        galp_destroy(ctx);
        galp_host_graph_free(g);
        return 1;
    }
    const double per_iter = st.iters_run ? st.device_ms / 1e3 / st.iters_run : 0.0;
    for (int i = 0; i < st.iters_run && i < GALP_MAX_ITERS; ++i)
        std::printf("%d: %f (s), updated %lld\n", i + 1, per_iter, (long long)st.updates[i]);

    double nmi = 0.0, fm = 0.0, ari = 0.0;
    if (argc == 4) {
        std::vector<int32_t> labels((size_t)g->n);
        galp_get_labels(ctx, labels.data(), g->n);
        const char *gt = argv[3];
        nmi = galp_nmi(gt, labels.data(), g->n);
        fm = galp_f_measure(gt, labels.data(), g->n);
        ari = galp_ari(gt, labels.data(), g->n);
    }
    galp_destroy(ctx);
    const char *filename = basename(argv[2]);
    std::fprintf(stderr, "%s\t%s\t%d\t%d\t%f\t%f\t%f\t%f\t%f\n", proc_name.c_str(), filename, niter, buffer_pow,
                 st.f1, st.f2, nmi, fm, ari);
    galp_host_graph_free(g);
    return 0;
}
