// Result formats of the reference, byte for byte in layout:
//   <prefix>_probtraj.csv   src/statistics/window_average_small.cpp:181-250
//   <prefix>_fp.csv         src/statistics/fixed_states.cu:154-187
//   <prefix>_final_states.csv  (no reference file: the reference prints its final-state
//                           histogram, final_states.cpp:53-66, only to stdout and leaves
//                           final_states::write_csv empty, final_states.cpp:68)
//   stdout report           final_states.cpp:53-66, fixed_states.cu:139-152,
//                           window_average_small.cpp:142-179, in the order of main.cpp:65-74
// Probabilities are computed in double from the exact fixed-point sums and printed through
// float with the default 6 significant digits, the type and precision the reference prints.
#include <cmath>
#include <fstream>
#include <iostream>

#include "sim.hpp"

namespace mbg {

std::string state_string(const std::vector<std::string>& names, const std::vector<uint32_t>& words, int n) {
    // state_t::to_string, src/state.cpp:29-47
    std::string s;
    bool first = true;
    for (int i = 0; i < n; ++i) {
        if ((words[i >> 5] >> (i & 31)) & 1u) {
            if (!first) s += " -- ";
            first = false;
            s += names[i];
        }
    }
    return s.empty() ? "<nil>" : s;
}

std::string out_state_string(const Sim& s, uint32_t idx) {
    // non_internal_idx_to_state, src/statistics/window_average_small.cpp:109-124
    std::vector<uint32_t> w(s.cm.words, 0u);
    for (int q = 0; q < s.cm.n_out; ++q)
        if ((idx >> q) & 1u) {
            int i = s.cm.out_nodes[q];
            w[i >> 5] |= 1u << (i & 31);
        }
    return state_string(s.names, w, s.cm.n);
}

// get_single_result_prob, window_average_small.cpp:126-140, for a bin with this raw sum
double window_prob(const Sim& s, uint64_t sum) {
    const double n = (double)s.n_traj;
    if (s.cm.discrete) return (double)sum / n;
    return ((double)sum / 4294967296.0) / (n * s.cm.tick);
}

double window_th(const Sim& s, int w) {
    double v = ((double)s.th[w] / 4294967296.0) / (double)s.n_traj;
    return s.cm.discrete ? v : v / s.cm.tick;
}

namespace {

// Walks the reached bins of window w only (the reference walks all 2^n_out states).
double window_entropy(const Sim& s, int w, int* nonzero) {
    double h = 0;
    int nz = 0;
    for (size_t e = s.wstart[w]; e < s.wstart[w + 1]; ++e) {
        double p = window_prob(s, s.wsum[e]);
        if ((float)p == 0.f) continue;
        ++nz;
        h += -std::log2(p) * p;
    }
    if (nonzero) *nonzero = nz;
    return h;
}

float window_start(const Sim& s, int w) { return (float)w * (float)s.cm.tick; }

}  // namespace

void write_probtraj_csv(const Sim& s, const std::string& path) {
    std::ofstream ofs(path);
    if (!ofs) throw IoError("cannot write " + path);
    const uint32_t smask = (uint32_t)(((uint64_t)1 << s.cm.n_out) - 1);
    int max_states = 0;
    for (int w = 0; w < s.cm.windows; ++w) {
        int nz = 0;
        window_entropy(s, w, &nz);
        max_states = std::max(max_states, nz);
    }
    ofs << "Time\tTH\tErrorTH\tH\tHD=0";
    for (int i = 0; i < max_states; ++i) ofs << "\tState\tProba\tErrorProba";
    ofs << "\n";
    for (int w = 0; w < s.cm.windows; ++w) {
        ofs << window_start(s, w) << "\t";
        ofs << (float)window_th(s, w) << "\t" << 0.f << "\t" << (float)window_entropy(s, w, nullptr) << "\t" << 0.f;
        for (size_t e = s.wstart[w]; e < s.wstart[w + 1]; ++e) {
            double p = window_prob(s, s.wsum[e]);
            if ((float)p == 0.f) continue;
            ofs << "\t" << out_state_string(s, s.wbin[e] & smask) << "\t" << (float)p << "\t" << 0.f;
        }
        ofs << "\n";
    }
    if (!ofs) throw IoError("error writing " + path);
}

void write_fp_csv(const Sim& s, const std::string& path) {
    std::ofstream ofs(path);
    if (!ofs) throw IoError("cannot write " + path);
    ofs << "Fixed Points (" << s.fixed.size() << ")\n";
    ofs << "FP\tProba\tState";
    for (auto& nm : s.names) ofs << "\t" << nm;
    ofs << "\n";
    int i_fp = 0;
    for (const FixedPoint& f : s.fixed) {
        ofs << "#" << i_fp << "\t" << (float)((double)f.count / (double)s.n_traj) << "\t"
            << state_string(s.names, f.words, s.cm.n);
        for (int i = 0; i < s.cm.n; ++i) ofs << "\t" << ((f.words[i >> 5] >> (i & 31)) & 1u);
        ofs << "\n";
        ++i_fp;
    }
    if (!ofs) throw IoError("error writing " + path);
}

// Final-state histogram in the layout of the fixed-point file: a count line, a header naming the
// output nodes, then one row per reached output state in increasing index order with its share of
// the trajectories and one 0/1 column per output node.
void write_final_states_csv(const Sim& s, const std::string& path) {
    std::ofstream ofs(path);
    if (!ofs) throw IoError("cannot write " + path);
    ofs << "Final States (" << s.fin_state.size() << ")\n";
    ofs << "Proba\tState";
    for (int q = 0; q < s.cm.n_out; ++q) ofs << "\t" << s.names[s.cm.out_nodes[q]];
    ofs << "\n";
    for (size_t e = 0; e < s.fin_state.size(); ++e) {
        const uint32_t x = s.fin_state[e];
        ofs << (float)((double)s.fin_count[e] / (double)s.n_traj) << "\t" << out_state_string(s, x);
        for (int q = 0; q < s.cm.n_out; ++q) ofs << "\t" << ((x >> q) & 1u);
        ofs << "\n";
    }
    if (!ofs) throw IoError("error writing " + path);
}

void print_results(const Sim& s, std::ostream& os) {
    const size_t S = (size_t)1 << s.cm.n_out;
    const uint32_t smask = (uint32_t)(S - 1);
    os << "final points:\n";
    for (size_t e = 0; e < s.fin_state.size(); ++e)
        os << (float)((double)s.fin_count[e] / (double)s.n_traj) << " " << out_state_string(s, s.fin_state[e]) << "\n";
    os << "fixed points:\n";
    for (const FixedPoint& f : s.fixed)
        os << (float)((double)f.count / (double)s.n_traj) << " " << state_string(s.names, f.words, s.cm.n) << "\n";
    for (int w = 0; w < s.cm.windows; ++w) {
        os << "window (" << window_start(s, w) << ", " << window_start(s, w + 1) << "]\n";
        os << "entropy: " << (float)window_entropy(s, w, nullptr) << "\n";
        os << "transition entropy: " << (float)window_th(s, w) << "\n";
        for (size_t e = s.wstart[w]; e < s.wstart[w + 1]; ++e) {
            double p = window_prob(s, s.wsum[e]);
            if ((float)p == 0.f) continue;
            os << (float)p << " " << out_state_string(s, s.wbin[e] & smask) << "\n";
        }
    }
    os.flush();
}

}  // namespace mbg
