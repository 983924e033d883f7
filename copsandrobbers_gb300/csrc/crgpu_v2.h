// crgpu_v2.h - the v2 (macro-turn) solver behind the C ABI.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "../../include/crgpu.h"

namespace crgpu {

struct V2Solver;

uint64_t v2_footprint(int n, int k, int p);
int v2_create(V2Solver** out, cudaStream_t st, int num_sms, int n, int k, int p,
              const uint32_t* d_rp, const uint16_t* d_col, const uint32_t* h_rp,
              const uint16_t* h_col, const uint32_t* d_binom, const uint16_t* d_configs,
              uint32_t C, std::string* err);
void v2_destroy(V2Solver* s);
int v2_init(V2Solver* s, uint64_t* caps, cr_solve_stats* stats, std::string* err);
int v2_pass(V2Solver* s, uint64_t* found, cr_solve_stats* stats, std::string* err);
void v2_verdict(V2Solver* s, unsigned long long* best_key);
const uint8_t* v2_table(const V2Solver* s);
cr_v2_hash_stats v2_hash_stats(const V2Solver* s);
int v2_set_hash_capacity(V2Solver* s, uint64_t slots, std::string* err);
// A solved single-plane table (C * n bytes, host memory) loaded as the store: the table
// uploaded and its marked plane rebuilt on the device.
int v2_load_states(V2Solver* s, const uint8_t* states, std::string* err);

}  // namespace crgpu
