// msm.cuh -- Pippenger MSM over prepared (precomputed-window) SRS layers.
#pragma once
#include <cstddef>
#include <cstdint>

#include "g1.cuh"
#include "host_ec.h"

struct HpCudaContext;

namespace hp {

// One prepared SRS layer: window w of point i is 2^(c*w) * P_i in affine
// Montgomery form at bases[w * n + i], so every window of a scalar's
// signed-digit expansion indexes the same 2^(c-1) buckets and no per-window
// combination is needed.  Built once by msm_prepare_layer().
//
// Scalar randomisation: the MSM is computed as sum (s_i + d_i) P_i - D with a
// fixed pseudo-random d per layer and D = sum d_i P_i precomputed at prepare
// time.  The value is the same group element; the bucket loads no longer
// depend on the scalars' distribution (an all-ones table -- frac and prod of
// an identity permutation -- would otherwise send every record to bucket 1).
struct MsmLayer {
    size_t n = 0;
    int c = 0;        // window bits
    int windows = 0;  // ceil(256 / c)
    Affine *bases = nullptr;  // windows * n points (device, context scratch)
    Fr *delta = nullptr;      // n canonical Fr < 2^254 (device), or null
    host::Xyzz64 minus_d{};   // -sum d_i P_i, added by the host finish
};

// Window width minimising ceil(256/c) * 10 n + 28 * 2^(c-1) for c in [4, 20]
// (mixed additions into buckets + two XYZZ additions per bucket to reduce).
int msm_window_bits(size_t n);
inline int msm_windows(int c) { return (256 + c - 1) / c; }

// Bucket reduction geometry: buckets are split into segments of `seg` and
// the segment sums combined by bit subsets (see msm.cu).
struct MsmShape {
    size_t buckets;  // 2^(c-1)
    size_t seg;      // buckets per segment
    size_t segments; // buckets / seg
    int seg_bits;    // log2(segments)
    int partials;    // seg_bits + 1 XYZZ outputs per MSM
};
MsmShape msm_shape(const MsmLayer &layer);

// Upload n 97-byte packets as window 0 and derive the other windows.
// Returns false if a packet is malformed (bad tag / non-canonical coordinate).
bool msm_prepare_layer(HpCudaContext *ctx, MsmLayer &layer, const uint8_t *packets, size_t n);
void msm_release_layer(HpCudaContext *ctx, MsmLayer &layer);
// A layer over the first n bases of `source` (its own window width, windows
// and randomiser), built from source's device-resident window 0.
void msm_prepare_prefix(HpCudaContext *ctx, MsmLayer &prefix, const MsmLayer &source, size_t n);

// Enqueue one MSM of the first `count` bases of the layer (all n when 0) with
// `count` Montgomery scalars; writes msm_shape(layer).partials XYZZ values to
// out_partials (device).  All work, scratch included, is ordered on `stream`
// (the context stream when null); no synchronisation.
void msm_run(HpCudaContext *ctx, const MsmLayer &layer, const Fr *scalars, Xyzz *out_partials,
             cudaStream_t stream = nullptr, size_t count = 0);

// Batch XYZZ -> affine (one field inversion per 512 points); pre: n Fq scratch.
void xyzz_to_affine(HpCudaContext *ctx, const Xyzz *in, Affine *out, Fq *pre, size_t n);

// Many MSMs in one launch per phase: task i = the first n points of layer
// `layer` with `scalars`; writes its msm_shape(layer).partials rows (what
// msm_run writes for it alone) to out_rows + out_row.
struct MsmTask {
    const MsmLayer *layer;
    const Fr *scalars;
    size_t n;
    size_t out_row;
};
void msm_run_many(HpCudaContext *ctx, const MsmTask *tasks, size_t count, Xyzz *out_rows,
                  cudaStream_t stream = nullptr);

// Host: combine the partials of one MSM into a point.
host::Xyzz64 msm_combine_host(const MsmShape &shape, const host::Xyzz64 *partials);
// Host: combine the partials of one MSM over `layer` (removing its
// randomisation offset) into its result point / a 97-byte G1 packet.
host::Xyzz64 msm_result_host(const MsmLayer &layer, const host::Xyzz64 *partials);
void msm_finalize_host(const MsmLayer &layer, const host::Xyzz64 *partials, uint8_t *out97);

}  // namespace hp
