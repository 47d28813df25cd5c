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
    // node0[p]: the first node t whose slot product p has (its slots are
    // t = node0[p] .. arity).  0 in round 1; 1 from round 2 on for products
    // of arity equal to the degree, whose t = 0 share of the message the
    // round's claim supplies: p(0) = claim - p(1), claim = p_prev(r_prev).
    uint8_t node0[kMaxProducts];
};

constexpr uint16_t kNoWriter = 0xffff;

// How a round is run (sumcheck.cu): the kernel family and, where it has one,
// its grid in blocks per SM (0: one thread per item of the round).
enum RouteKernel : uint8_t {
    kRouteNone = 0,
    kRouteOneBlock = 1,   // one block, (factor, pair) then (product, pair) items (<= 64 pairs)
    kRoutePerPair = 2,    // one pair per thread, per-thread slot sums in shared memory
    kRouteSlot = 3,       // (slot, pair) items, separate fold pass
    kRouteSlotFused = 4,  // (slot, pair) items folding their own factors
    kRoutePp = 5,         // (product, pair) items, separate fold pass
    kRoutePpFused = 6,    // (product, pair) items folding their own factors
    kRouteTiled = 7,      // shared-memory tiles staged by bulk copies, fold + (slot, pair) items
    kRouteEq = 8,         // zero-check states: (node, pair) items of the polynomial without its eq factor
    kRouteKinds = 9
};
struct RoundRoute {
    uint8_t kernel;
    uint8_t per_sm;
};
// Tuning key of a round: ceil(log2 pairs), the largest product arity, the
// slot count (sum over products of arity + 1) and whether the round folds
// the previous challenge in (every round but the first).
struct RoundKey {
    int log2_pairs;
    int max_arity;
    int slots;
    int fold;
    bool operator<(const RoundKey &o) const {
        if (log2_pairs != o.log2_pairs) return log2_pairs < o.log2_pairs;
        if (max_arity != o.max_arity) return max_arity < o.max_arity;
        if (slots != o.slots) return slots < o.slots;
        return fold < o.fold;
    }
};
inline int ceil_log2_size(size_t x) {
    int k = 0;
    while ((size_t(1) << k) < x) k++;
    return k;
}
// The process-wide table of measured round routes (tune.cu: it shares the
// MSM tuning table's file, built-in GB300 entries and environment override).
bool sumcheck_route_lookup(const RoundKey &key, RoundRoute &out);
void sumcheck_route_store(const RoundKey &key, const RoundRoute &route, double us);

}  // namespace hp
