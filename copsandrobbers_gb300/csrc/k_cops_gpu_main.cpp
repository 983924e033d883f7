// k_cops_gpu_main.cpp - driver for a solver translation unit, with the reference driver's
// argv, phase order, failure messages and timing report (app/main.cpp:20-111;
// lib/src/Profiler.cpp:43-123 for the report layout its harness parses).
#include <chrono>
#include <iomanip>
#include <iostream>
#include <map>
#include <string>
#include <vector>

bool loadGraphFile(const char* filename, int k, int p);
bool buildAuxGraph();
bool initializeCaptures();
bool mainLoop();
bool findFinalResult();
bool outputData();

#include CR_SOLVER_TU

namespace {

class PhaseClock {
   public:
    PhaseClock() : start_(now()), mark_(start_) {}
    void enter(const std::string& name) {
        const double t = now();
        if (!current_.empty()) totals_[current_] += t - mark_;
        if (!totals_.count(name)) {
            order_.push_back(name);
            totals_[name] = 0.0;
        }
        current_ = name;
        mark_ = t;
    }
    void print() {
        const double t = now();
        if (!current_.empty()) totals_[current_] += t - mark_;
        current_.clear();
        const double app = t - start_;
        double tracked = 0;
        for (auto& kv : totals_) tracked += kv.second;
        size_t width = 0;
        for (auto& s : order_) width = std::max(width, std::string("  -> " + s + " ").size());
        auto row = [&](const std::string& label, double sec, size_t align) {
            size_t dashes = align > label.size() + 2 ? align - label.size() - 2 : 1;
            std::cout << "||" << label << std::string(dashes, '-') << "=> " << std::right << std::fixed
                      << std::setprecision(4) << std::setw(12) << sec << " s (" << std::setprecision(2)
                      << std::setw(6) << (app > 0 ? 100.0 * sec / app : 0.0) << "%)\n";
        };
        std::cout << "\n||>>>>>=====-----=====<<<<<     Timing Profiler Report     >>>>>=====-----=====<<<<<\n||\n";
        row("   Total App Uptime ", app, 37);
        row("    -> Tracked Execution ", tracked, 32);
        std::cout << "||\n||\n||  ---===<<<>>>===---   Drill Down   ---===<<<>>>===---\n||\n";
        for (auto& s : order_) row("  -> " + s + " ", totals_[s], width + 3);
        std::cout << "||\n||>>>>>>>>>>>>>>>>================------------------================<<<<<<<<<<<<<<<<\n\n";
    }

   private:
    static double now() {
        return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
    }
    double start_, mark_;
    std::string current_;
    std::vector<std::string> order_;
    std::map<std::string, double> totals_;
};

void solveCopsAndRobbers(const char* filename, int k, int p) {
    PhaseClock prof;
    struct Phase {
        const char* name;
        bool (*fn)();
    };
    prof.enter("Load Graph File");
    if (loadGraphFile(filename, k, p)) {
        std::cout << "[FAILED STEP]: 'Load Graph File' was unsuccessful!\n";
        return;
    }
    prof.enter("Idle");
    const Phase phases[] = {{"Build Aux Graph", buildAuxGraph},
                            {"Initialize Captures", initializeCaptures},
                            {"Main Loop", mainLoop},
                            {"Find Final Result", findFinalResult},
                            {"Output Data", outputData}};
    for (const Phase& ph : phases) {
        prof.enter(ph.name);
        if (ph.fn()) {
            std::cout << "[FAILED STEP]: '" << ph.name << "' was unsuccessful!\n";
            return;
        }
        prof.enter("Idle");
    }
    prof.print();
}

}  // namespace

int main(int argc, char* argv[]) {
    if (argc < 3 || argc > 4) {
        std::cout << "Usage: " << argv[0] << " <graph_file.txt> <num_cops> [visibility_p]\n";
        std::cout << "Example (1/2 Vis): " << argv[0] << " graph3.txt 4 2\n";
        std::cout << "Example (Standard): " << argv[0] << " graph3.txt 4\n";
        return 1;
    }
    const int k = std::stoi(argv[2]);
    const int p = argc == 4 ? std::stoi(argv[3]) : 1;
    solveCopsAndRobbers(argv[1], k, p);
    return 0;
}
