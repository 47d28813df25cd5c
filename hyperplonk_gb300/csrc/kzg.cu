// kzg.cu -- multilinear-KZG prepared parameters, commit, multi_commit, open.
//
// Reference: backend/src/cpu/multilinear_kzg.rs:40-137 (semantics) and
// backend/src/ascend910b3/native/bridge_kzg.cpp:253-676 (ABI behaviour).
//  - params hold num_vars + 1 SRS layers; layer k has 2^(num_vars - k) bases
//    and is prepared once (Montgomery affine + precomputed MSM windows) and
//    stays resident in HBM;
//  - commit(poly with nv vars) = MSM against layer (num_vars - nv);
//  - open runs nv rounds of q[b] = f[2b+1] - f[2b], f[b] = f[2b] + q[b]*z_i
//    (one fused kernel) and an MSM of q against layer (num_vars - nv + 1 + i);
//    quotients stay on the device as MSM scalars, only the partial sums and
//    the final scalar come back.
#include <algorithm>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <map>
#include <vector>

#include "host_ec.h"
#include "kzg.cuh"
#include "mle.cuh"
#include "msm.cuh"
#include "runtime.cuh"

using hp::check_cuda;
using hp::check_launch;
using hp::fail;
using hp::Fr;
using hp::guard;
using hp::require;

namespace hp {

__global__ void k_open_fold(const Fr *f, Fr *fnext, Fr *q, size_t half, Fr z) {
    for (size_t b = blockIdx.x * size_t(blockDim.x) + threadIdx.x; b < half;
         b += size_t(gridDim.x) * blockDim.x) {
        Fr lo = load_fr(&f[2 * b]);
        Fr d = load_fr(&f[2 * b + 1]) - lo;
        store_fr(&q[b], d);
        store_fr(&fnext[b], lo + d * z);
    }
}

static const MsmLayer &ready_layer(const HpCudaMultilinearKzgPreparedProverParam *p, size_t k) {
    if (k >= p->layers.size() || !p->uploaded[k]) fail(HP_CUDA_STATUS_INVALID_STATE);
    return p->layers[k];
}

// Download `total` XYZZ partials and finish each MSM into a packet.
// Independent MSMs, task i writing its partial rows at the running offset.
// MSMs whose scalars are all 0 or 1 are sums of bases (msm_run_binary, a
// worker stream each).  Of the others, MSMs of >= 4 M (point,
// window) records fill the GPU alone: one msm_run each, overlapped on worker
// streams; all smaller ones share one launch per phase (msm_run_many) on
// another worker stream (msm_runs_alone).
static void run_msms(HpCudaContext *ctx, std::vector<MsmTask> tasks, Xyzz *parts) {
    if (tasks.empty()) return;
    size_t o = 0;
    for (auto &t : tasks) {
        t.out_row = o;
        o += size_t(msm_shape(*t.layer).partials);
    }
    std::vector<uint64_t> ones;
    const std::vector<char> binary = msm_binary_tasks(ctx, tasks.data(), tasks.size(), &ones);
    std::vector<MsmTask> big, small, sums;
    std::vector<char> mostly_ones;
    for (size_t i = 0; i < tasks.size(); i++) {
        const MsmTask &t = tasks[i];
        (binary[i] ? sums : msm_runs_alone(size_t(t.layer->windows) * t.n) ? big : small).push_back(t);
        if (binary[i]) mostly_ones.push_back(char(2 * ones[i] > t.n));
    }
    std::stable_sort(big.begin(), big.end(), [](const MsmTask &a, const MsmTask &b) { return a.n > b.n; });
    const size_t lanes = big.size() + (small.empty() ? 0 : 1) + sums.size();
    const int k = int(std::min<size_t>(lanes, HpCudaContext::kWorkers));
    ctx->fork(k);
    size_t w = 0;
    // sums of bases end in a latency-bound tree: one worker stream each, so the tails overlap
    for (size_t i = 0; i < sums.size(); i++) {
        const MsmTask &t = sums[i];
        msm_run_binary(ctx, *t.layer, t.scalars, t.n, parts + t.out_row, ctx->workers[w++ % size_t(k)],
                       mostly_ones[i] != 0);
    }
    if (!small.empty()) msm_run_many(ctx, small.data(), small.size(), parts, ctx->workers[w++ % size_t(k)]);
    for (const auto &t : big) msm_run(ctx, *t.layer, t.scalars, parts + t.out_row, ctx->workers[w++ % size_t(k)], t.n);
    ctx->join(k);
}

// One MSM over the whole layer on the context stream: a sum of bases when
// every scalar is 0 or 1, else msm_run.
static void run_one_msm(HpCudaContext *ctx, const MsmLayer &layer, const Fr *scalars, Xyzz *parts) {
    const MsmTask task{&layer, scalars, layer.n, 0};
    std::vector<uint64_t> ones;
    if (msm_binary_tasks(ctx, &task, 1, &ones)[0])
        msm_run_binary(ctx, layer, scalars, layer.n, parts, nullptr, 2 * ones[0] > layer.n);
    else msm_run(ctx, layer, scalars, parts);
}

static void finish_msms(HpCudaContext *ctx, const Xyzz *dev, const std::vector<const MsmLayer *> &layers,
                        uint8_t *out97) {
    std::vector<MsmShape> shapes;
    for (auto *l : layers) shapes.push_back(msm_shape(*l));
    size_t total = 0;
    for (auto &s : shapes) total += size_t(s.partials);
    std::vector<host::Xyzz64> hostp(std::max<size_t>(total, 1));
    if (total)
        check_cuda(cudaMemcpyAsync(hostp.data(), dev, total * sizeof(Xyzz), cudaMemcpyDeviceToHost, ctx->stream));
    ctx->sync();
    // every result's Horner chain (spread over the context's host threads),
    // then one inversion for all affine conversions
    std::vector<host::Xyzz64> results(shapes.size());
    std::vector<size_t> offs(shapes.size());
    size_t off = 0;
    for (size_t i = 0; i < shapes.size(); i++) {
        offs[i] = off;
        off += size_t(shapes[i].partials);
    }
    ctx->host_parallel_for(shapes.size(), [&](size_t i) {
        results[i] = msm_result_host(*layers[i], hostp.data() + offs[i]);
    });
    host::xyzz_to_packets(results.data(), results.size(), out97);
}

}  // namespace hp

extern "C" HpCudaStatus hp_cuda_v1_multilinear_kzg_params_create(
    HpCudaContext *ctx, size_t num_vars, HpCudaMultilinearKzgPreparedProverParam **out) {
    if (out) *out = nullptr;
    return guard([&] {
        hp::require_ctx(ctx);
        require(out != nullptr && num_vars <= hp::kMaxNumVars);
        auto *p = new HpCudaMultilinearKzgPreparedProverParam();
        p->num_vars = num_vars;
        p->layers.resize(num_vars + 1);
        p->uploaded.assign(num_vars + 1, false);
        *out = p;
    });
}

extern "C" HpCudaStatus hp_cuda_v1_multilinear_kzg_params_upload_layer(
    HpCudaContext *ctx, HpCudaMultilinearKzgPreparedProverParam *params, size_t layer_index,
    const uint8_t *points, size_t point_count) {
    return guard([&] {
        hp::require_ctx(ctx);
        require(params != nullptr && points != nullptr && layer_index <= params->num_vars);
        require(point_count == hp::table_len(params->num_vars - layer_index));
        require(!params->uploaded[layer_index]);
        hp::MsmLayer layer;
        bool ok;
        try {
            ok = hp::msm_prepare_layer(ctx, layer, points, point_count);
        } catch (...) {
            hp::msm_release_layer(ctx, layer);
            throw;
        }
        if (!ok) {
            hp::msm_release_layer(ctx, layer);
            fail(HP_CUDA_STATUS_INVALID_PARAMETERS);
        }
        params->layers[layer_index] = layer;
        params->uploaded[layer_index] = true;
    });
}

extern "C" HpCudaStatus hp_cuda_v1_multilinear_kzg_params_destroy(
    HpCudaContext *ctx, HpCudaMultilinearKzgPreparedProverParam *params) {
    return guard([&] {
        hp::require_ctx(ctx);
        require(params != nullptr);
        for (auto &l : params->layers) hp::msm_release_layer(ctx, l);
        for (auto &kv : params->prefixes) hp::msm_release_layer(ctx, kv.second);
        delete params;
    });
}

extern "C" HpCudaStatus hp_cuda_v1_multilinear_kzg_commit(
    HpCudaContext *ctx, const HpCudaMultilinearKzgPreparedProverParam *params,
    HpCudaDeviceAddress polynomial, size_t num_vars, uint8_t *out_commitment) {
    return guard([&] {
        hp::require_ctx(ctx);
        require(params != nullptr && out_commitment != nullptr && num_vars <= params->num_vars);
        const Fr *scalars = hp::mle_ptr(ctx, polynomial, num_vars);
        const hp::MsmLayer &layer = hp::ready_layer(params, params->num_vars - num_vars);
        hp::MsmShape sh = hp::msm_shape(layer);
        hp::Scratch parts(ctx, size_t(sh.partials) * sizeof(hp::Xyzz));
        hp::run_one_msm(ctx, layer, scalars, parts.as<hp::Xyzz>());
        hp::finish_msms(ctx, parts.as<hp::Xyzz>(), {&layer}, out_commitment);
    });
}

extern "C" HpCudaStatus hp_cuda_v1_multilinear_kzg_multi_commit(
    HpCudaContext *ctx, const HpCudaMultilinearKzgPreparedProverParam *params,
    const HpCudaDeviceAddress *polynomials, const size_t *num_vars, size_t count,
    uint8_t *out_commitments) {
    return guard([&] {
        hp::require_ctx(ctx);
        require(params != nullptr);
        if (count == 0) return;
        require(polynomials != nullptr && num_vars != nullptr && out_commitments != nullptr);
        std::vector<const Fr *> scalars(count);
        std::vector<const hp::MsmLayer *> layers(count);
        std::vector<hp::MsmShape> shapes(count);
        size_t total = 0;
        for (size_t i = 0; i < count; i++) {
            require(num_vars[i] <= params->num_vars);
            scalars[i] = hp::mle_ptr(ctx, polynomials[i], num_vars[i]);
            layers[i] = &hp::ready_layer(params, params->num_vars - num_vars[i]);
            shapes[i] = hp::msm_shape(*layers[i]);
            total += size_t(shapes[i].partials);
        }
        hp::Scratch parts(ctx, total * sizeof(hp::Xyzz));
        std::vector<hp::MsmTask> tasks(count);
        for (size_t i = 0; i < count; i++) tasks[i] = hp::MsmTask{layers[i], scalars[i], layers[i]->n, 0};
        hp::run_msms(ctx, tasks, parts.as<hp::Xyzz>());
        hp::finish_msms(ctx, parts.as<hp::Xyzz>(), layers, out_commitments);
    });
}

extern "C" HpCudaStatus hp_cuda_v1_multilinear_kzg_open(
    HpCudaContext *ctx, const HpCudaMultilinearKzgPreparedProverParam *params,
    HpCudaDeviceAddress polynomial, size_t num_vars, const uint8_t *point, uint8_t *out_quotients,
    uint8_t *out_evaluation) {
    return guard([&] {
        hp::require_ctx(ctx);
        require(params != nullptr && out_evaluation != nullptr && num_vars <= params->num_vars);
        require(num_vars == 0 || (point != nullptr && out_quotients != nullptr));
        const Fr *f = hp::mle_ptr(ctx, polynomial, num_vars);
        std::vector<Fr> z(num_vars);
        for (size_t i = 0; i < num_vars; i++) z[i] = hp::host_scalar(point + 32 * i);
        if (num_vars == 0) {
            hp::download_canonical(ctx, f, 1, out_evaluation);
            return;
        }
        const size_t nv = num_vars, ignored = params->num_vars - nv + 1;
        std::vector<const hp::MsmLayer *> layers(nv);
        std::vector<hp::MsmShape> shapes(nv);
        size_t total = 0;
        for (size_t i = 0; i < nv; i++) {
            layers[i] = &hp::ready_layer(params, ignored + i);
            shapes[i] = hp::msm_shape(*layers[i]);
            total += size_t(shapes[i].partials);
        }
        hp::Scratch parts(ctx, total * sizeof(hp::Xyzz));
        hp::Scratch fa(ctx, hp::table_len(nv - 1) * sizeof(Fr));
        hp::Scratch fb(ctx, hp::table_len(nv >= 2 ? nv - 2 : 0) * sizeof(Fr));
        // all quotients first (q_i at offset 2^nv - 2^(nv-i)), then their MSMs
        // together (run_msms): the late rounds' MSMs are tiny and latency
        // bound one at a time
        hp::Scratch q(ctx, hp::table_len(nv) * sizeof(Fr));
        const Fr *cur = f;
        Fr *bufs[2] = {fa.as<Fr>(), fb.as<Fr>()};
        std::vector<size_t> q_off(nv);
        size_t qo = 0;
        for (size_t i = 0; i < nv; i++) {
            size_t half = hp::table_len(nv - 1 - i);
            Fr *next = bufs[i & 1];
            q_off[i] = qo;
            hp::k_open_fold<<<hp::grid_for(ctx, half, 256), 256, 0, ctx->stream>>>(cur, next, q.as<Fr>() + qo,
                                                                                   half, z[i]);
            check_launch();
            qo += half;
            cur = next;
        }
        std::vector<hp::MsmTask> tasks(nv);
        for (size_t i = 0; i < nv; i++) tasks[i] = hp::MsmTask{layers[i], q.as<Fr>() + q_off[i], layers[i]->n, 0};
        hp::run_msms(ctx, tasks, parts.as<hp::Xyzz>());
        hp::download_canonical(ctx, cur, 1, out_evaluation);
        hp::finish_msms(ctx, parts.as<hp::Xyzz>(), layers, out_quotients);
    });
}

extern "C" HpCudaStatus hp_cuda_v1_msm(HpCudaContext *ctx, const uint8_t *bases, const uint8_t *scalars,
                                       size_t count, uint8_t *out_point) {
    return guard([&] {
        hp::require_ctx(ctx);
        require(out_point != nullptr);
        if (count == 0) {
            std::memset(out_point, 0, 97);
            out_point[0] = 1;
            return;
        }
        require(bases != nullptr && scalars != nullptr && count < (size_t(1) << 27));
        hp::MsmLayer layer;
        struct Release {
            HpCudaContext *c;
            hp::MsmLayer *l;
            ~Release() { hp::msm_release_layer(c, *l); }
        } release{ctx, &layer};
        if (!hp::msm_prepare_layer(ctx, layer, bases, count)) fail(HP_CUDA_STATUS_INVALID_PARAMETERS);
        hp::Scratch s(ctx, count * sizeof(Fr));
        ctx->clear_flags();
        check_cuda(cudaMemcpyAsync(s.ptr, scalars, count * sizeof(Fr), cudaMemcpyHostToDevice, ctx->stream));
        hp::mle_to_mont_checked(ctx, s.as<Fr>(), count);
        if (ctx->sync_flags() & hp::kFlagNonCanonical) fail(HP_CUDA_STATUS_INVALID_PARAMETERS);
        hp::MsmShape sh = hp::msm_shape(layer);
        hp::Scratch parts(ctx, size_t(sh.partials) * sizeof(hp::Xyzz));
        hp::run_one_msm(ctx, layer, s.as<Fr>(), parts.as<hp::Xyzz>());
        hp::finish_msms(ctx, parts.as<hp::Xyzz>(), {&layer}, out_point);
    });
}

extern "C" HpCudaStatus hp_cuda_v1_batch_msm(HpCudaContext *ctx, HpCudaMultilinearKzgPreparedProverParam *params,
                                             size_t layer_index, const HpCudaDeviceAddress *scalars,
                                             const size_t *num_vars, size_t count, uint8_t *out_points) {
    return guard([&] {
        hp::require_ctx(ctx);
        require(params != nullptr);
        if (count == 0) return;
        require(scalars != nullptr && num_vars != nullptr && out_points != nullptr);
        const hp::MsmLayer &base = hp::ready_layer(params, layer_index);
        std::vector<const Fr *> sc(count);
        std::vector<const hp::MsmLayer *> layers(count);
        size_t total = 0;
        for (size_t i = 0; i < count; i++) {
            const size_t n = hp::table_len(num_vars[i]);
            require(num_vars[i] <= hp::kMaxNumVars && n <= base.n);
            sc[i] = hp::mle_ptr(ctx, scalars[i], num_vars[i]);
            if (n == base.n) {
                layers[i] = &base;
            } else {
                auto key = std::make_pair(layer_index, n);
                auto it = params->prefixes.find(key);
                if (it == params->prefixes.end()) {
                    hp::MsmLayer pl;
                    try {
                        hp::msm_prepare_prefix(ctx, pl, base, n);
                    } catch (...) {
                        hp::msm_release_layer(ctx, pl);
                        throw;
                    }
                    it = params->prefixes.emplace(key, pl).first;
                }
                layers[i] = &it->second;
            }
            total += size_t(hp::msm_shape(*layers[i]).partials);
        }
        hp::Scratch parts(ctx, total * sizeof(hp::Xyzz));
        std::vector<hp::MsmTask> tasks(count);
        for (size_t i = 0; i < count; i++) tasks[i] = hp::MsmTask{layers[i], sc[i], layers[i]->n, 0};
        hp::run_msms(ctx, tasks, parts.as<hp::Xyzz>());
        hp::finish_msms(ctx, parts.as<hp::Xyzz>(), layers, out_points);
    });
}
