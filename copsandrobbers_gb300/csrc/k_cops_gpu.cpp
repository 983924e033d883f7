// k_cops_gpu.cpp - drop-in solver translation unit for the reference's six-phase contract
// (app/main.cpp:11-16).  It is included by a driver the way the reference includes a solver
// (app/main.cpp:18, `#include ALGORITHM_INCLUDE`), and runs the solve on the GPU through the
// C ABI of libcrgpu.so.  stdout lines and the cache table file match the reference solvers
// (solvers/k_cops_visibility.cpp and, with CR_GPU_RULES=2, solvers/k_cops_visibility_v2.cpp),
// so the reference's sweep harness (util/test_k_cops_visibility.py) parses it unchanged.
//
// Phase return convention as in the reference: false = success, true = failure.
#include <sys/stat.h>

#include <cstdint>
#include <cstdio>
#include <cstring>
#include <iomanip>
#include <iostream>
#include <string>
#include <vector>

#include "crgpu.h"

#ifndef CR_GPU_RULES
#define CR_GPU_RULES CR_RULES_V1
#endif

namespace crdrop {

const char* g_file = nullptr;
int g_k = 0, g_p = 0, g_columns = 0;
std::vector<uint32_t> g_row_ptr;
std::vector<uint16_t> g_col;
int32_t g_n = 0;
cr_context* g_ctx = nullptr;
cr_solver* g_solver = nullptr;
uint64_t g_host_bytes = 0;

inline std::string algo_name() {
    return (CR_GPU_RULES == CR_RULES_V2 ? std::string("k_cops_v2_") : std::string("k_cops_")) +
           std::to_string(g_p) + "vis";
}

// cache/<algo>__<graph stem>__<k>-cops__<p>-vis__00__auxgraph.bin (CacheManager.h:16-26).
inline std::string cache_path() {
    std::string name = g_file ? g_file : "";
    size_t slash = name.find_last_of("/\\");
    if (slash != std::string::npos) name = name.substr(slash + 1);
    size_t dot = name.find_last_of('.');
    if (dot != std::string::npos && dot > 0) name = name.substr(0, dot);
    mkdir("cache", 0755);
    return "cache/" + algo_name() + "__" + name + "__" + std::to_string(g_k) + "-cops__" +
           std::to_string(g_p) + "-vis__00__auxgraph.bin";
}

inline bool report(int rc, const char* what) {
    if (rc == CR_OK) return false;
    std::cerr << "Error: " << what << ": " << cr_context_last_error(g_ctx) << " (code " << rc << ")\n";
    return true;
}

// The reference's "Memory Tracking Report" line that its harness parses
// (lib/src/Allocator.cpp:69-209; util/test_k_cops_visibility.py:83).
inline void print_footprint() {
    uint64_t dev = cr_solver_footprint(g_n, g_k, g_p, CR_GPU_RULES);
    uint64_t total = dev + g_host_bytes;
    auto line = [](const char* label, uint64_t b) {
        std::string s = std::string("||") + label;
        size_t pad = s.size() < 40 ? 40 - s.size() : 1;
        std::cout << s << std::string(pad, '-') << "=> " << std::setw(12) << b << " B / " << std::fixed
                  << std::setprecision(2) << std::setw(8) << b / 1048576.0 << " MB / " << std::setw(5)
                  << b / 1073741824.0 << " GB\n";
    };
    std::cout << "\n||>>>>>=====-----=====<<<<<     Memory Tracking Report     >>>>>=====-----=====<<<<<\n||\n";
    line("   Total Footprint ", total);
    line("    -> GPU State Store ", dev);
    line("    -> Host Graph ", g_host_bytes);
    std::cout << "||>>>>>>>>>>>>>>>>================------------------================<<<<<<<<<<<<<<<<\n\n";
}

}  // namespace crdrop

bool loadGraphFile(const char* filename_param, int k_param, int p_param) {
    using namespace crdrop;
    g_file = filename_param;
    g_k = k_param;
    g_p = p_param;
    g_columns = CR_GPU_RULES == CR_RULES_V2 ? 1 : 2 * p_param;
    FILE* f = std::fopen(filename_param, "rb");
    std::vector<char> text;
    if (f) {
        std::fseek(f, 0, SEEK_END);
        long len = std::ftell(f);
        std::fseek(f, 0, SEEK_SET);
        if (len > 0) {
            text.resize((size_t)len);
            if (std::fread(text.data(), 1, text.size(), f) != text.size()) text.clear();
        }
        std::fclose(f);
    }
    size_t nnz = 0;
    if (text.empty() || cr_graph_parse(text.data(), text.size(), &g_n, nullptr, nullptr, 0, &nnz) != CR_OK ||
        g_n == 0) {
        std::cerr << "Error: Graph is empty or failed to load.\n";
        return 1;
    }
    g_row_ptr.assign(g_n + 1, 0);
    g_col.assign(nnz ? nnz : 1, 0);
    if (cr_graph_parse(text.data(), text.size(), &g_n, g_row_ptr.data(), g_col.data(), g_col.size(), &nnz) != CR_OK) {
        std::cerr << "Error: Graph is empty or failed to load.\n";
        return 1;
    }
    g_host_bytes = (uint64_t)g_row_ptr.size() * 4 + (uint64_t)g_col.size() * 2;
    return 0;
}

bool buildAuxGraph() {
    using namespace crdrop;
    if (!g_ctx && cr_context_create(0, nullptr, &g_ctx) != CR_OK) {
        std::cerr << "Error: no usable CUDA device.\n";
        return 1;
    }
    cr_graph g{g_n, g_row_ptr.data(), g_col.data()};
    if (report(cr_solver_create(g_ctx, &g, g_k, g_p, CR_GPU_RULES, &g_solver), "Unable to generate aux graph"))
        return 1;
    // CacheManager::loadAuxGraph (CacheManager.h:78-141): a table file under the same key whose
    // header matches (self-edge flags 0/0 in words 6-7) is a hit, and it is read into the device
    // store (the key, sizes, sections and configs are checked as the reference checks them; v1
    // and v2 alike).  initializeCaptures resets every column either way, so a hit and a miss
    // solve identically.
    bool hit = false;
    if (FILE* f = std::fopen(cache_path().c_str(), "rb")) {
        uint64_t h[12];
        hit = std::fread(h, 8, 12, f) == 12 && h[6] == 0 && h[7] == 0;
        std::fclose(f);
        if (hit) hit = cr_solver_load_table_file(g_solver, cache_path().c_str()) == CR_OK;
    }
    if (hit) {
        std::cout << "Loaded AuxGraph from cache!\n";
    } else if (CR_GPU_RULES == CR_RULES_V2) {
        std::cout << "Cache miss. Creating new AuxGraph (single-plane state space)...\n";
    } else {
        std::cout << "Cache miss. Creating new AuxGraph with " << g_columns << " columns...\n";
    }
    if (!hit) {
        cr_table_sizes sz;
        cr_solver_sizes(g_solver, &sz);
        std::cout << "Building AuxGraph transition table for " << sz.config_count << " configurations...\n";
        uint64_t total = 0;
        if (report(cr_solver_build_transitions(g_solver, &total), "transition table")) return 1;
        std::cout << "Transitions generated. Total edge pointers: " << total << "\n";
    }
    return 0;
}

bool initializeCaptures() {
    using namespace crdrop;
    uint64_t caps = 0;
    if (report(cr_solver_init(g_solver, &caps), "initializeCaptures")) return 1;
    std::cout << "Initialized " << caps << " base captures.\n";
    return 0;
}

bool mainLoop() {
    using namespace crdrop;
    if (CR_GPU_RULES == CR_RULES_V2)
        std::cout << "Starting Macro-Turn Trajectory Search for " << g_p << "-Visibility...\n";
    else
        std::cout << "Starting Backward Induction Loop for " << g_p << "-Visibility...\n";
    for (int pass = 1;; ++pass) {
        uint64_t found = 0;
        if (report(cr_solver_pass(g_solver, &found), "mainLoop")) return 1;
        std::cout << "Pass " << pass << ": Found " << found << " new winning states.\n";
        if (found == 0) break;
    }
    return 0;
}

bool findFinalResult() {
    using namespace crdrop;
    std::cout << "\n--- FINAL VERDICT ---\n";
    cr_verdict v;
    if (report(cr_solver_verdict(g_solver, &v), "findFinalResult")) return 1;
    if (v.win) {
        std::cout << "RESULT: WIN. " << g_k << " Cop(s) CAN win this graph with 1/" << g_p << " visibility.\n";
        std::cout << "Optimal Cop Start Positions: (";
        for (int i = 0; i < g_k; ++i) std::cout << (int)v.positions[i] << (i == g_k - 1 ? "" : ", ");
        std::cout << ")\n";
        if (CR_GPU_RULES == CR_RULES_V2)
            std::cout << "Capture Time: " << v.capture_plies << " plys.\n";
        else
            std::cout << "Capture Time: " << v.capture_plies << " plys (" << (v.capture_plies / g_columns)
                      << " full cycles).\n";
    } else {
        std::cout << "RESULT: LOSS. " << g_k << " Cop(s) CANNOT guarantee a win.\n";
        std::cout << "(The Robber has a strategy to survive indefinitely against any start).\n";
    }
    print_footprint();
    return 0;
}

bool outputData() {
    using namespace crdrop;
    std::cout << "Saving filled AuxGraph to cache... ";
    if (g_n > 256 || cr_solver_write_table_file(g_solver, cache_path().c_str()) != CR_OK) {
        std::cout << "Failed!\n";
        return 1;
    }
    std::cout << "Success!\n";
    cr_solver_destroy(g_solver);
    g_solver = nullptr;
    cr_context_destroy(g_ctx);
    g_ctx = nullptr;
    return 0;
}
