// msm.cuh -- Pippenger MSM over prepared (precomputed-window) SRS layers.
#pragma once
#include <cstddef>
#include <cstdint>
#include <vector>

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
    uint32_t seg = 0;    // buckets per reduction segment, 0: the size rule in msm_shape
    uint32_t chunk = 0;  // records per accumulation chunk, 0: the size rule
    Affine *bases = nullptr;  // windows * n points (device, context scratch)
    Fr *delta = nullptr;      // n canonical Fr < 2^254 (device), or null
    host::Xyzz64 minus_d{};   // -sum d_i P_i, added by the host finish
    Xyzz *d_sum = nullptr;    // D = sum d_i P_i (device, one point), or null
    Xyzz *base_sum = nullptr; // sum of the n window-0 bases (device, one point)
};

// Window width for a new layer of n points: HP_MSM_WINDOW_BITS, else the
// tuning table, else msm_window_bits_model(n).
int msm_window_bits(size_t n);
// Window width minimising ceil(256/c) * 10 n + 28 * 2^(c-1) for c in [4, 20]
// (mixed additions into buckets + two XYZZ additions per bucket to reduce).
int msm_window_bits_model(size_t n);
inline int msm_windows(int c) { return (256 + c - 1) / c; }
// Whether window width c (4..22) suits an MSM of n points: records fit in 31
// bits and the top window piles at most 2048 records onto a bucket.
bool msm_window_fits(size_t n, int c);

// Measured MSM geometry (csrc/tune.cu).  Entries are keyed by ceil(log2 n)
// for an MSM run alone (window width, segment length, chunk length) and by
// ceil(log2 records) for a many-MSM launch (chunk length); a zero field means
// "no entry, use the size rule".  Process-wide, guarded by a mutex.
struct MsmTuning {
    int c = 0;
    uint32_t seg = 0;
    uint32_t chunk = 0;
};
MsmTuning msm_tuning_alone(size_t n);
uint32_t msm_tuning_many_chunk(size_t records);
// window width, segment and chunk from the tuning table for a layer of n points
void msm_apply_tuning(MsmLayer &layer);
// the size rule's reduction segment for 2^(c-1) buckets / accumulation chunk
// for an MSM of `records` (window, point) records
uint32_t msm_default_seg(int c);
uint32_t msm_default_chunk(size_t records);
// largest number of reduction segments one MSM may have (subset blocks)
size_t msm_max_segments();

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
// The same with a given window width (4..22), for the autotuner.
void msm_prepare_prefix_c(HpCudaContext *ctx, MsmLayer &prefix, const MsmLayer &source, size_t n, int c);
// Rebuild windows 1..W-1 and the randomiser of a prepared layer whose window
// width the tuning table changed (window 0 is kept); seg and chunk follow it.
void msm_retune_layer(HpCudaContext *ctx, MsmLayer &layer);
// n pseudo-random Montgomery scalars from `seed` on `stream` (autotuner input).
void msm_random_scalars(HpCudaContext *ctx, Fr *out, size_t n, uint64_t seed, cudaStream_t stream);

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
// `chunk` forces the accumulation chunk length (the autotuner); 0 takes the
// layer's tuned chunk for a launch of one MSM, the tuning table's entry for
// the launch's record count for several, else the size rule.
void msm_run_many(HpCudaContext *ctx, const MsmTask *tasks, size_t count, Xyzz *out_rows,
                  cudaStream_t stream = nullptr, uint32_t chunk = 0);
// Whether an MSM of `records` (window, point) records runs alone (msm_run,
// on a worker stream) rather than in a launch shared with the other small
// MSMs of a call (msm_run_many): from 2^22 records on, where one MSM fills
// the GPU.  HP_MSM_MANY=0 runs every MSM alone, HP_MSM_MANY=1 none.
bool msm_runs_alone(size_t records);
// Limits of one many-MSM launch (larger task lists are split into groups).
constexpr size_t kMsmManyMaxInstances = 64;
constexpr size_t kMsmManyMaxRecords = size_t(1) << 27;
// The chunk length an accumulation of `records` records runs with, given a
// tuned value (0: none): HP_ACC_CHUNK, else the tuned value, else the size rule.
uint32_t msm_effective_chunk(size_t records, uint32_t tuned);

// Binary scalars.  An MSM whose scalars are all 0 or 1 (the product-check
// tables frac and prod of a circuit whose permutation is the identity) is
// the sum of the selected bases: one mixed addition per 1 instead of one per
// (point, window) record.  msm_binary_tasks classifies every task of a call
// in one launch and one synchronisation (HP_MSM_BINARY=0: none is binary);
// msm_run_binary writes the same partial rows msm_run would combine to (all
// but the last at infinity, the last = the sum + D so that the host finish,
// which adds -D, is unchanged).
// `ones`, when given, receives each task's number of scalars equal to 1.
// With `complement` (a whole layer, n = layer.n, most scalars 1) the sum is
// formed as the layer's base_sum minus the bases of the zero scalars.
std::vector<char> msm_binary_tasks(HpCudaContext *ctx, const MsmTask *tasks, size_t count,
                                   std::vector<uint64_t> *ones = nullptr);
void msm_run_binary(HpCudaContext *ctx, const MsmLayer &layer, const Fr *scalars, size_t n, Xyzz *out_partials,
                    cudaStream_t stream = nullptr, bool complement = false);

// Host: combine the partials of one MSM into a point.
host::Xyzz64 msm_combine_host(const MsmShape &shape, const host::Xyzz64 *partials);
// Host: combine the partials of one MSM over `layer` (removing its
// randomisation offset) into its result point / a 97-byte G1 packet.
host::Xyzz64 msm_result_host(const MsmLayer &layer, const host::Xyzz64 *partials);
void msm_finalize_host(const MsmLayer &layer, const host::Xyzz64 *partials, uint8_t *out97);

}  // namespace hp
