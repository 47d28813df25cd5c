// kzg.cuh -- the prepared multilinear-KZG parameter object behind the C ABI
// (shared by kzg.cu and the MSM autotuner in tune.cu).
#pragma once
#include <cstddef>
#include <map>
#include <utility>
#include <vector>

#include "msm.cuh"

// num_vars + 1 SRS layers (layer k: 2^(num_vars - k) bases), each prepared
// once and resident in HBM.
struct HpCudaMultilinearKzgPreparedProverParam {
    size_t num_vars = 0;
    std::vector<hp::MsmLayer> layers;
    std::vector<bool> uploaded;
    // prefix layers for batched MSMs over the first n bases of layer k,
    // keyed by (k, n), built on first use
    std::map<std::pair<size_t, size_t>, hp::MsmLayer> prefixes;
};
