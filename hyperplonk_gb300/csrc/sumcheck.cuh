// sumcheck.cuh -- product description of a virtual polynomial as it rides in
// kernel parameters: sum_p c_p * prod_{j in product p} factor_j.  Mirrors the
// reference's ABI product encoding (backend/src/ascend910b3/sum_check.rs:32-90:
// coefficients, offsets, indices over identity-deduplicated factors).
#pragma once
#include <cstdint>

#include "field.cuh"

namespace hp {

constexpr int kMaxProducts = 64;
constexpr int kMaxIndices = 1024;
constexpr int kMaxDegree = 64;
constexpr int kMaxFactors = 32;  // distinct factor tables of one state

struct SumcheckDesc {
    int factor_count;
    int product_count;
    int slot_count;  // sum over products of (arity + 1)
    int max_arity;
    uint16_t offsets[kMaxProducts + 1];
    uint16_t slot_base[kMaxProducts];
    uint8_t indices[kMaxIndices];
    // writer[f]: the position in `indices` of factor f's first occurrence
    // (kNoWriter if f is in no product); the wide round kernel's item at that
    // position and t = 0 stores f's folded pair
    uint16_t writer[kMaxFactors];
};

constexpr uint16_t kNoWriter = 0xffff;

}  // namespace hp
