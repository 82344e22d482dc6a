// MaBoSSG command line, a thin client of the libmbg C ABI.
//
// Same surface as src/main.cpp:101-169: `MaBoSSG [-o prefix] bnd_file cfg_file`; any other
// argument count prints the usage line and returns 1; without -o the results go to stdout in the
// reference's report format, with -o they go to <prefix>_probtraj.csv and <prefix>_fp.csv. More
// than 20 output nodes is an error (main.cpp:142-146). The node-count limit MAX_NODES
// (main.cpp:148-152) is lifted to the library's own limits.
//
// Environment (the argument list stays the reference's): MBG_DEVICE (CUDA ordinal),
// MBG_LAYOUT (auto | thread | warp | lane | lane_global), MBG_TIMINGS=1 (JSON run summary on stderr),
// MBG_CONFIG_EXPR (cfg statements applied after the cfg file, e.g. "$k = 2; max_time = 50;"),
// MBG_MUTANTS (comma-separated NODE:ON / NODE:OFF clamps), MBG_FINAL_STATES_CSV=1 (with -o,
// also <prefix>_final_states.csv).
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <string>
#include <vector>

#include "../../../include/mbg.h"

int main(int argc, char** argv) {
    std::vector<std::string> args(argv + 1, argv + argc);
    if (!(args.size() == 2 || (args.size() == 4 && args[0] == "-o"))) {
        std::cout << "Usage: MaBoSSG [-o prefix] bnd_file cfg_file" << std::endl;
        return 1;
    }
    std::string prefix, bnd = args[0], cfg = args[1];
    if (args[0] == "-o") {
        prefix = args[1];
        bnd = args[2];
        cfg = args[3];
    }
    mbg_model* model = nullptr;
    if (mbg_model_parse_files_overrides(bnd.c_str(), cfg.c_str(), std::getenv("MBG_CONFIG_EXPR"), &model) != MBG_OK) {
        std::cerr << mbg_last_error() << std::endl;
        return 1;
    }
    if (const char* mu = std::getenv("MBG_MUTANTS"); mu && *mu) {
        mbg_model_info mi;
        mbg_model_info_get(model, &mi);
        std::vector<int32_t> nodes, values;
        std::string spec(mu), bad;
        size_t pos = 0;
        while (pos <= spec.size() && bad.empty()) {
            size_t end = spec.find(',', pos);
            if (end == std::string::npos) end = spec.size();
            std::string item = spec.substr(pos, end - pos);
            pos = end + 1;
            if (item.empty()) continue;
            size_t colon = item.rfind(':');
            std::string name = colon == std::string::npos ? item : item.substr(0, colon);
            std::string val = colon == std::string::npos ? "" : item.substr(colon + 1);
            int32_t idx = -1;
            for (int32_t i = 0; i < mi.nodes; ++i)
                if (name == mbg_model_node_name(model, i)) idx = i;
            if (idx < 0 || (val != "ON" && val != "OFF")) {
                bad = item;
                break;
            }
            nodes.push_back(idx);
            values.push_back(val == "ON" ? 1 : 0);
        }
        mbg_model* mutant = nullptr;
        if (!bad.empty()) {
            std::cerr << "MBG_MUTANTS: cannot read '" << bad << "' (expected NODE:ON or NODE:OFF)" << std::endl;
        } else if (mbg_model_with_mutations(model, nodes.data(), values.data(), (int32_t)nodes.size(), &mutant) !=
                   MBG_OK) {
            std::cerr << mbg_last_error() << std::endl;
        }
        mbg_model_destroy(model);
        if (!mutant) return 1;
        model = mutant;
    }
    mbg_model_info info;
    mbg_model_info_get(model, &info);
    if (info.outputs > 20) {
        std::cerr << "This executable supports a maximum of 20 non-internal nodes." << std::endl;
        mbg_model_destroy(model);
        return 1;
    }
    mbg_sim_opts opts;
    mbg_sim_opts_default(&opts);
    if (const char* d = std::getenv("MBG_DEVICE")) opts.device = std::atoi(d);
    if (const char* l = std::getenv("MBG_LAYOUT")) {
        if (!std::strcmp(l, "thread")) opts.layout = MBG_LAYOUT_THREAD;
        else if (!std::strcmp(l, "warp")) opts.layout = MBG_LAYOUT_WARP;
        else if (!std::strcmp(l, "lane")) opts.layout = MBG_LAYOUT_LANE;
        else if (!std::strcmp(l, "lane_global")) opts.layout = MBG_LAYOUT_LANE_GLOBAL;
    }
    mbg_sim* sim = nullptr;
    int rc = 0;
    if (mbg_sim_create(model, &opts, &sim) != MBG_OK || mbg_sim_run(sim, nullptr) != MBG_OK) {
        std::cerr << mbg_last_error() << std::endl;
        rc = 1;
    } else {
        mbg_status st = prefix.empty()
                            ? mbg_print_results(sim, "-")
                            : (mbg_write_probtraj_csv(sim, prefix.c_str()) == MBG_OK
                                   ? mbg_write_fp_csv(sim, prefix.c_str())
                                   : MBG_ERR_IO);
        const char* fs = std::getenv("MBG_FINAL_STATES_CSV");
        if (st == MBG_OK && !prefix.empty() && fs && *fs == '1') st = mbg_write_final_states_csv(sim, prefix.c_str());
        if (st != MBG_OK) {
            std::cerr << mbg_last_error() << std::endl;
            rc = 1;
        }
        const char* t = std::getenv("MBG_TIMINGS");
        if (t && *t == '1') {
            mbg_run_summary s;
            mbg_sim_summary(sim, &s);
            std::fprintf(stderr,
                         "{\"trajectories\": %llu, \"transitions\": %llu, \"fixed_points\": %llu, "
                         "\"sim_ms\": %.3f, \"jit_ms\": %.3f, \"transitions_per_s\": %.6g, \"layout\": %d}\n",
                         (unsigned long long)s.trajectories, (unsigned long long)s.transitions,
                         (unsigned long long)s.fixed_points, s.sim_ms, s.jit_ms,
                         s.sim_ms > 0 ? s.transitions / (s.sim_ms * 1e-3) : 0.0, s.layout);
        }
    }
    mbg_sim_destroy(sim);
    mbg_model_destroy(model);
    return rc;
}
