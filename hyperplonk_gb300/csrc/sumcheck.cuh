// sumcheck.cuh -- product description of a virtual polynomial as it rides in
// kernel parameters: sum_p c_p * prod_{j in product p} factor_j.  Mirrors the
// reference's ABI product encoding (backend/src/ascend910b3/sum_check.rs:32-90:
// coefficients, offsets, indices over identity-deduplicated factors).
#pragma once
#include <cstdint>

#include "field.cuh"

namespace hp {

constexpr int kMaxProducts = 64;
constexpr int kMaxIndices = 256;
constexpr int kMaxDegree = 64;

struct SumcheckDesc {
    int factor_count;
    int product_count;
    int slot_count;  // sum over products of (arity + 1)
    int max_arity;
    uint16_t offsets[kMaxProducts + 1];
    uint16_t slot_base[kMaxProducts];
    uint8_t indices[kMaxIndices];
};

}  // namespace hp
