// gpet_cli.cpp - `gpet input_PET.in [key=value ...]`, the drop-in for
// `./gPET input_PET.in` (main.cu:26-276): reads the same configuration and
// data/ tables (relative to the working directory), simulates, and appends the
// output records to ./output/ as the reference does. key=value arguments set
// the options of gpet_set_option (seed, n_decays, coinc_window_ns, ...).
#include <cstdio>
#include <cstring>
#include <string>

#include "gpet.h"

int main(int argc, char** argv)
{
    if (argc < 2) {
        std::printf("Please execute ./gpet input_file [key=value ...]\n");
        return 1;
    }
    gpet_ctx* ctx = nullptr;
    int rc = gpet_create(0, &ctx);
    if (rc) {
        std::fprintf(stderr, "gpet: no usable CUDA device (%d)\n", rc);
        return 1;
    }
    std::string out_dir = "./output";
    for (int i = 2; i < argc; ++i) {
        const char* eq = std::strchr(argv[i], '=');
        if (!eq) { std::fprintf(stderr, "gpet: expected key=value, got %s\n", argv[i]); return 1; }
        std::string key(argv[i], eq - argv[i]);
        if (key == "out_dir") { out_dir = eq + 1; continue; }
        if (gpet_set_option(ctx, key.c_str(), eq + 1)) {
            std::fprintf(stderr, "gpet: %s\n", gpet_last_error(ctx));
            return 1;
        }
    }
    if ((rc = gpet_load_config(ctx, argv[1]))) {
        std::fprintf(stderr, "gpet: %s\n", gpet_last_error(ctx));
        return 1;
    }
    gpet_run_stats st;
    if ((rc = gpet_run(ctx, &st))) {
        std::fprintf(stderr, "gpet: %s\n", gpet_last_error(ctx));
        return 1;
    }
    std::printf("decays %lld pairs %lld entered %lld pulses %lld hits %lld\n", (long long)st.n_decays,
                (long long)st.n_pairs, (long long)st.n_entered, (long long)st.n_pulses, (long long)st.n_hits);
    std::printf("counts after thresholder %lld, after deadtime %lld, singles %lld\n", (long long)st.n_threshold,
                (long long)st.n_deadtime, (long long)st.n_singles);
    std::printf("coincidences %lld (true %lld scatter %lld random %lld, multiples %lld)\n", (long long)st.n_coinc,
                (long long)st.n_true, (long long)st.n_scatter, (long long)st.n_random, (long long)st.n_multiple);
    std::printf("Simulation time: %f s (device)\n", st.ms_total * 1e-3);
    if ((rc = gpet_write_outputs(ctx, out_dir.c_str()))) {
        std::fprintf(stderr, "gpet: %s\n", gpet_last_error(ctx));
        return 1;
    }
    gpet_destroy(ctx);
    return 0;
}
