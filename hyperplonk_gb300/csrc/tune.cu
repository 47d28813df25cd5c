// tune.cu -- MSM autotuner: measured geometry per MSM size and per batch mix.
//
// The MSM (msm.cu) has three free parameters whose best values depend on
// the size, the batch mix and the part: the window width c (how many
// precomputed windows and buckets), the reduction segment length (bucket
// chains of 2 seg dependent additions vs. the number of subset sums) and the
// accumulation chunk length L (records per thread: longer chains vs. more
// fix-up pieces and fewer chunks to fill 152 SMs).  msm.cu has a size rule
// for each; this file measures them instead:
//
//  - mode 0 (one MSM on its own), keyed by ceil(log2 n): coordinate descent
//    from the size rule's choice -- window widths c0-4..c0+2, then segment
//    lengths seg/4..seg*4, then chunk lengths 4..64 -- each candidate timed
//    as the median of a few runs with CUDA events on the context stream,
//    over pseudo-random scalars and the first n bases of the parameters'
//    layer 0, on the path the library takes for that size (msm_run from 2^22
//    records on, else a launch of msm_run_many holding this one MSM);
//  - mode 1 (one many-MSM launch over a mix of sizes), keyed by
//    ceil(log2 records): the chunk length of the shared accumulation launch.
//
// A candidate is kept only when it is at least 1% faster than the best so
// far.  Every candidate's result point is compared with the size rule's (a
// geometry change must not change the group element): a mismatch is an
// InvalidState failure and leaves the table unchanged.
//
// The table is process-wide and starts from the entries measured on a GB300
// (msm_tuning_gb300.inc) when the current device has that name.  Layers
// prepared after an entry exists use it;
// hp_cuda_v1_msm_autotune also re-prepares the layers of the parameter object
// it ran on and drops that object's cached prefix layers.  Entries persist as
// a small text file (hp_cuda_v1_msm_tuning_save / _load, or the file named by
// HP_CUDA_MSM_TUNING, read at the first lookup):
//
//     hp_cuda msm tuning 1
//     device <name, spaces as _>
//     alone <log2 n> <c> <seg> <chunk> <ms>
//     many <log2 records> <chunk> <ms>
//     round <log2 pairs> <max arity> <slots> <fold 0/1> <kernel> <blocks per SM> <us>
//
// The last kind holds the sumcheck round routes that
// hp_cuda_v1_sumcheck_autotune measures (sumcheck.cu): which round kernel
// and grid run a round of that many pairs and that product shape.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <memory>
#include <mutex>
#include <sstream>
#include <string>
#include <vector>

#include "kzg.cuh"
#include "msm.cuh"
#include "runtime.cuh"
#include "sumcheck.cuh"

namespace hp {
namespace {

struct AloneEntry {
    MsmTuning t;
    double ms;
};
struct ManyEntry {
    uint32_t chunk;
    double ms;
};

struct RouteEntry {
    RoundRoute route;
    double us;
};

struct TuningTable {
    std::mutex mu;
    std::map<int, AloneEntry> alone;  // ceil(log2 n)
    std::map<int, ManyEntry> many;    // ceil(log2 records)
    std::map<RoundKey, RouteEntry> rounds;
    std::string device = "any";
    bool env_checked = false;
};

struct Parsed {
    std::map<int, AloneEntry> alone;
    std::map<int, ManyEntry> many;
    std::map<RoundKey, RouteEntry> rounds;
    std::string device = "any";
};

TuningTable &table() {
    static TuningTable t;
    return t;
}

int ceil_log2(size_t x) {
    int k = 0;
    while ((size_t(1) << k) < x) k++;
    return k;
}

std::string device_token(const char *name) {
    std::string s = name && name[0] ? name : "any";
    for (char &ch : s)
        if (ch == ' ' || ch == '\t' || ch == '\n' || ch == '\r') ch = '_';
    return s;
}

bool valid_seg(long v) { return v >= 1 && v <= 64 && (v & (v - 1)) == 0; }
bool valid_chunk(long v) { return v >= 2 && v <= 1024; }

// Parse a tuning table; false on any malformed line (nothing is applied
// then).
bool parse_table(std::istream &in, Parsed &out) {
    std::string line;
    if (!std::getline(in, line) || line != "hp_cuda msm tuning 1") return false;
    out = Parsed();
    while (std::getline(in, line)) {
        if (line.empty()) continue;
        std::istringstream ls(line);
        std::string kind;
        ls >> kind;
        if (kind == "device") {
            if (!(ls >> out.device)) return false;
        } else if (kind == "alone") {
            long k, c, seg, chunk;
            double ms;
            if (!(ls >> k >> c >> seg >> chunk >> ms)) return false;
            if (k < 0 || k > 40 || c < 4 || c > 22 || !valid_seg(seg) || !valid_chunk(chunk) || !std::isfinite(ms) ||
                ms < 0)
                return false;
            MsmTuning t;
            t.c = int(c);
            t.seg = uint32_t(seg);
            t.chunk = uint32_t(chunk);
            out.alone[int(k)] = AloneEntry{t, ms};
        } else if (kind == "many") {
            long k, chunk;
            double ms;
            if (!(ls >> k >> chunk >> ms)) return false;
            if (k < 0 || k > 40 || !valid_chunk(chunk) || !std::isfinite(ms) || ms < 0) return false;
            out.many[int(k)] = ManyEntry{uint32_t(chunk), ms};
        } else if (kind == "round") {
            // round <ceil log2 pairs> <max arity> <slots> <fold> <kernel> <blocks per SM> <us>
            long k, arity, slots, fold, kernel, per_sm;
            double us;
            if (!(ls >> k >> arity >> slots >> fold >> kernel >> per_sm >> us)) return false;
            if (k < 0 || k > 40 || arity < 1 || arity > kMaxDegree || slots < 1 || slots > 4096 ||
                (fold != 0 && fold != 1) || kernel <= kRouteNone || kernel >= kRouteKinds || per_sm < 0 ||
                per_sm > 64 || !std::isfinite(us) || us < 0)
                return false;
            out.rounds[RoundKey{int(k), int(arity), int(slots), int(fold)}] =
                RouteEntry{RoundRoute{uint8_t(kernel), uint8_t(per_sm)}, us};
        } else {
            return false;
        }
        std::string extra;
        if (ls >> extra) return false;
    }
    return true;
}

bool parse_file(const char *path, Parsed &out) {
    std::ifstream in(path);
    return in && parse_table(in, out);
}

void merge_into(TuningTable &t, const Parsed &p) {
    for (auto &kv : p.alone) t.alone[kv.first] = kv.second;
    for (auto &kv : p.many) t.many[kv.first] = kv.second;
    for (auto &kv : p.rounds) t.rounds[kv.first] = kv.second;
    t.device = p.device;
}

// The table measured on a GB300 (msm_tuning_gb300.inc), the default on
// devices of that name.
const char kBuiltinGb300[] =
#include "msm_tuning_gb300.inc"
    ;

// Name of the current CUDA device as a table token, or "" without one.
std::string current_device_token() {
    int dev = 0;
    cudaDeviceProp prop;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaGetDeviceProperties(&prop, dev) != cudaSuccess) {
        (void)cudaGetLastError();
        return std::string();
    }
    return device_token(prop.name);
}

// At the first lookup: the built-in table when the current device has its
// name, then the file named by HP_CUDA_MSM_TUNING over it (an unreadable or
// malformed file is ignored); HP_CUDA_MSM_TUNING=off leaves the table empty
// (the size rules).
void load_env_locked(TuningTable &t) {
    if (t.env_checked) return;
    t.env_checked = true;
    const char *path = std::getenv("HP_CUDA_MSM_TUNING");
    if (path && std::strcmp(path, "off") == 0) return;
    Parsed parsed;
    std::istringstream builtin(kBuiltinGb300);
    if (parse_table(builtin, parsed) && parsed.device == current_device_token()) merge_into(t, parsed);
    if (!path || !path[0]) return;
    if (!parse_file(path, parsed)) return;
    merge_into(t, parsed);
}

bool geometry_env_set() {
    return std::getenv("HP_MSM_WINDOW_BITS") || std::getenv("HP_MSM_SEG") || std::getenv("HP_ACC_CHUNK");
}

struct EventPair {
    cudaEvent_t a = nullptr, b = nullptr;
    EventPair() {
        check_cuda(cudaEventCreate(&a));
        check_cuda(cudaEventCreate(&b));
    }
    ~EventPair() {
        if (a) cudaEventDestroy(a);
        if (b) cudaEventDestroy(b);
    }
};

// Median device time of `reps` calls of run() on the context stream, after
// one untimed call.
template <class Run>
double median_ms(HpCudaContext *ctx, int reps, Run &&run) {
    EventPair ev;
    run();
    std::vector<float> ms;
    for (int r = 0; r < reps; r++) {
        check_cuda(cudaEventRecord(ev.a, ctx->stream));
        run();
        check_cuda(cudaEventRecord(ev.b, ctx->stream));
        check_cuda(cudaEventSynchronize(ev.b));
        float x = 0;
        check_cuda(cudaEventElapsedTime(&x, ev.a, ev.b));
        ms.push_back(x);
    }
    std::sort(ms.begin(), ms.end());
    return double(ms[ms.size() / 2]);
}

int reps_for(size_t records) { return records < (size_t(1) << 22) ? 7 : 3; }

// The finished point(s) of MSM partial rows already on the device.
std::vector<uint8_t> finish_points(HpCudaContext *ctx, const Xyzz *dev, const std::vector<const MsmLayer *> &layers) {
    size_t total = 0;
    for (auto *l : layers) total += size_t(msm_shape(*l).partials);
    std::vector<host::Xyzz64> hostp(total);
    check_cuda(cudaMemcpyAsync(hostp.data(), dev, total * sizeof(Xyzz), cudaMemcpyDeviceToHost, ctx->stream));
    ctx->sync();
    std::vector<uint8_t> out(layers.size() * kG1PacketBytes);
    size_t off = 0;
    for (size_t i = 0; i < layers.size(); i++) {
        msm_finalize_host(*layers[i], hostp.data() + off, out.data() + i * kG1PacketBytes);
        off += size_t(msm_shape(*layers[i]).partials);
    }
    return out;
}

struct LayerGuard {
    HpCudaContext *ctx;
    MsmLayer layer;
    explicit LayerGuard(HpCudaContext *c) : ctx(c) {}
    ~LayerGuard() { msm_release_layer(ctx, layer); }
    LayerGuard(const LayerGuard &) = delete;
    LayerGuard &operator=(const LayerGuard &) = delete;
};

constexpr size_t kMaxPartialRows = 64;  // seg_bits + 1 <= 64 for any fitting geometry

// Mode 0: tune an MSM of n points over the first n bases of `source`, run
// the way the library runs it alone: msm_run from 2^22 records on, else a
// shared launch holding this one MSM (msm_runs_alone).
HpCudaMsmTuning tune_alone(HpCudaContext *ctx, const MsmLayer &source, size_t n) {
    Scratch scalars(ctx, n * sizeof(Fr)), parts(ctx, kMaxPartialRows * sizeof(Xyzz));
    msm_random_scalars(ctx, scalars.as<Fr>(), n, 0x7475e5eedull ^ uint64_t(n), ctx->stream);
    auto run_once = [&](MsmLayer &l, uint32_t chunk) {
        l.chunk = chunk;
        if (msm_runs_alone(size_t(l.windows) * n)) {
            msm_run(ctx, l, scalars.as<Fr>(), parts.as<Xyzz>(), ctx->stream, n);
        } else {
            const MsmTask task{&l, scalars.as<Fr>(), n, 0};
            msm_run_many(ctx, &task, 1, parts.as<Xyzz>(), ctx->stream, chunk);
        }
    };
    auto result = [&](const MsmLayer &l) { return finish_points(ctx, parts.as<Xyzz>(), {&l}); };

    // the size rule's geometry first: the reference point and time
    const int c0 = msm_window_bits_model(n);
    auto best = std::make_unique<LayerGuard>(ctx);
    msm_prepare_prefix_c(ctx, best->layer, source, n, c0);
    const int reps = reps_for(size_t(best->layer.windows) * n);
    uint32_t chunk = msm_default_chunk(size_t(best->layer.windows) * n);
    const double model_ms = median_ms(ctx, reps, [&] { run_once(best->layer, chunk); });
    const std::vector<uint8_t> ref = result(best->layer);
    double best_ms = model_ms;

    // 1. window width (each candidate is its own window table)
    for (int c = std::max(4, c0 - 4); c <= std::min(22, c0 + 2); c++) {
        if (c == c0 || !msm_window_fits(n, c)) continue;
        auto cand = std::make_unique<LayerGuard>(ctx);
        msm_prepare_prefix_c(ctx, cand->layer, source, n, c);
        const uint32_t ch = msm_default_chunk(size_t(cand->layer.windows) * n);
        const double ms = median_ms(ctx, reps, [&] { run_once(cand->layer, ch); });
        if (result(cand->layer) != ref) fail(HP_CUDA_STATUS_INVALID_STATE);
        if (ms < 0.99 * best_ms) {
            best_ms = ms;
            best = std::move(cand);
            chunk = ch;
        }
    }
    MsmLayer &L = best->layer;
    // 2. reduction segment length
    const uint32_t seg0 = uint32_t(msm_shape(L).seg);
    const size_t buckets = size_t(1) << (L.c - 1);
    for (uint32_t seg : {seg0 / 4, seg0 / 2, seg0 * 2, seg0 * 4}) {
        if (!valid_seg(long(seg)) || seg > buckets || buckets / seg > msm_max_segments()) continue;
        const uint32_t keep = L.seg;
        L.seg = seg;
        const double ms = median_ms(ctx, reps, [&] { run_once(L, chunk); });
        if (result(L) != ref) fail(HP_CUDA_STATUS_INVALID_STATE);
        if (ms < 0.99 * best_ms) best_ms = ms;
        else L.seg = keep;
    }
    // 3. accumulation chunk length
    for (uint32_t ch : {4u, 8u, 16u, 32u, 64u}) {
        if (ch == chunk) continue;
        const double ms = median_ms(ctx, reps, [&] { run_once(L, ch); });
        if (result(L) != ref) fail(HP_CUDA_STATUS_INVALID_STATE);
        if (ms < 0.99 * best_ms) {
            best_ms = ms;
            chunk = ch;
        }
    }
    HpCudaMsmTuning out{};
    out.size = n;
    out.mode = 0;
    out.window_bits = uint32_t(L.c);
    out.segment = uint32_t(msm_shape(L).seg);
    out.chunk = chunk;
    out.model_ms = model_ms;
    out.tuned_ms = best_ms;
    return out;
}

// Mode 1: tune the chunk length of one many-MSM launch over `tasks`.
HpCudaMsmTuning tune_many(HpCudaContext *ctx, const std::vector<MsmTask> &tasks_in, size_t records) {
    std::vector<MsmTask> tasks = tasks_in;
    std::vector<const MsmLayer *> layers;
    size_t rows = 0;
    for (auto &t : tasks) {
        t.out_row = rows;
        rows += size_t(msm_shape(*t.layer).partials);
        layers.push_back(t.layer);
    }
    Scratch parts(ctx, rows * sizeof(Xyzz));
    auto run_once = [&](uint32_t chunk) {
        msm_run_many(ctx, tasks.data(), tasks.size(), parts.as<Xyzz>(), ctx->stream, chunk);
    };
    const int reps = reps_for(records);
    const uint32_t chunk0 = msm_effective_chunk(records, 0);
    const double model_ms = median_ms(ctx, reps, [&] { run_once(chunk0); });
    const std::vector<uint8_t> ref = finish_points(ctx, parts.as<Xyzz>(), layers);
    double best_ms = model_ms;
    uint32_t best = chunk0;
    for (uint32_t chunk : {4u, 8u, 16u, 32u, 64u}) {
        if (chunk == chunk0) continue;
        const double ms = median_ms(ctx, reps, [&] { run_once(chunk); });
        if (finish_points(ctx, parts.as<Xyzz>(), layers) != ref) fail(HP_CUDA_STATUS_INVALID_STATE);
        if (ms < 0.99 * best_ms) {
            best_ms = ms;
            best = chunk;
        }
    }
    HpCudaMsmTuning out{};
    out.size = records;
    out.mode = 1;
    out.chunk = best;
    out.model_ms = model_ms;
    out.tuned_ms = best_ms;
    return out;
}

}  // namespace

MsmTuning msm_tuning_alone(size_t n) {
    TuningTable &t = table();
    std::lock_guard<std::mutex> lock(t.mu);
    load_env_locked(t);
    auto it = t.alone.find(ceil_log2(n));
    return it == t.alone.end() ? MsmTuning{} : it->second.t;
}

uint32_t msm_tuning_many_chunk(size_t records) {
    TuningTable &t = table();
    std::lock_guard<std::mutex> lock(t.mu);
    load_env_locked(t);
    auto it = t.many.find(ceil_log2(records));
    return it == t.many.end() ? 0u : it->second.chunk;
}

}  // namespace hp

using hp::fail;
using hp::guard;
using hp::require;

extern "C" HpCudaStatus hp_cuda_v1_msm_autotune(HpCudaContext *ctx, HpCudaMultilinearKzgPreparedProverParam *params,
                                                const size_t *num_vars, size_t count, int32_t mode,
                                                HpCudaMsmTuning *out) {
    return guard([&] {
        hp::require_ctx(ctx);
        require(params != nullptr && (count == 0 || (num_vars != nullptr && out != nullptr)));
        require(mode == 0 || mode == 1);
        if (count == 0) return;
        if (params->layers.empty() || !params->uploaded[0]) fail(HP_CUDA_STATUS_INVALID_STATE);
        // a geometry override in the environment would silently replace the candidates
        if (hp::geometry_env_set()) fail(HP_CUDA_STATUS_INVALID_STATE);
        const hp::MsmLayer &source = params->layers[0];
        for (size_t i = 0; i < count; i++)
            require(num_vars[i] <= hp::kMaxNumVars && hp::table_len(num_vars[i]) <= source.n);
        cudaDeviceProp prop;
        hp::check_cuda(cudaGetDeviceProperties(&prop, ctx->device));
        const std::string device = hp::device_token(prop.name);

        if (mode == 0) {
            std::vector<HpCudaMsmTuning> res(count);
            for (size_t i = 0; i < count; i++) res[i] = hp::tune_alone(ctx, source, hp::table_len(num_vars[i]));
            {
                hp::TuningTable &t = hp::table();
                std::lock_guard<std::mutex> lock(t.mu);
                hp::load_env_locked(t);
                for (const auto &r : res) {
                    hp::MsmTuning m;
                    m.c = int(r.window_bits);
                    m.seg = r.segment;
                    m.chunk = r.chunk;
                    t.alone[hp::ceil_log2(size_t(r.size))] = hp::AloneEntry{m, r.tuned_ms};
                }
                t.device = device;
            }
            // the parameter object follows the new entries; its prefix layers are rebuilt on use
            for (auto &kv : params->prefixes) hp::msm_release_layer(ctx, kv.second);
            params->prefixes.clear();
            for (size_t k = 0; k < params->layers.size(); k++)
                if (params->uploaded[k]) hp::msm_retune_layer(ctx, params->layers[k]);
            ctx->sync();
            std::copy(res.begin(), res.end(), out);
            return;
        }

        // mode 1: one launch over all sizes, each a prefix layer of layer 0 as batch_msm builds it
        require(count <= hp::kMsmManyMaxInstances);
        std::vector<std::unique_ptr<hp::LayerGuard>> keep;
        std::vector<hp::MsmTask> tasks(count);
        std::vector<std::unique_ptr<hp::Scratch>> scalars;
        size_t records = 0;
        for (size_t i = 0; i < count; i++) {
            const size_t n = hp::table_len(num_vars[i]);
            const hp::MsmLayer *layer = &source;
            if (n != source.n) {
                keep.push_back(std::make_unique<hp::LayerGuard>(ctx));
                hp::msm_prepare_prefix(ctx, keep.back()->layer, source, n);
                layer = &keep.back()->layer;
            }
            scalars.push_back(std::make_unique<hp::Scratch>(ctx, n * sizeof(hp::Fr)));
            hp::msm_random_scalars(ctx, scalars.back()->as<hp::Fr>(), n, 0x6d616e79ull + i, ctx->stream);
            tasks[i] = hp::MsmTask{layer, scalars.back()->as<hp::Fr>(), n, 0};
            records += size_t(layer->windows) * n;
        }
        require(records <= hp::kMsmManyMaxRecords);
        const HpCudaMsmTuning r = hp::tune_many(ctx, tasks, records);
        {
            hp::TuningTable &t = hp::table();
            std::lock_guard<std::mutex> lock(t.mu);
            hp::load_env_locked(t);
            t.many[hp::ceil_log2(records)] = hp::ManyEntry{r.chunk, r.tuned_ms};
            t.device = device;
        }
        ctx->sync();
        out[0] = r;
    });
}

extern "C" HpCudaStatus hp_cuda_v1_msm_tuning_query(int32_t mode, size_t size, uint32_t *out3) {
    return guard([&] {
        require(out3 != nullptr && (mode == 0 || mode == 1) && size >= 1);
        if (mode == 0) {
            hp::MsmLayer l;
            l.n = size;
            l.c = hp::msm_window_bits(size);
            l.windows = hp::msm_windows(l.c);
            hp::msm_apply_tuning(l);
            out3[0] = uint32_t(l.c);
            out3[1] = uint32_t(hp::msm_shape(l).seg);
            out3[2] = hp::msm_effective_chunk(size_t(l.windows) * size, l.chunk);
        } else {
            out3[0] = 0;
            out3[1] = 0;
            out3[2] = hp::msm_effective_chunk(size, hp::msm_tuning_many_chunk(size));
        }
    });
}

namespace hp {

bool sumcheck_route_lookup(const RoundKey &key, RoundRoute &out) {
    TuningTable &t = table();
    std::lock_guard<std::mutex> lock(t.mu);
    load_env_locked(t);
    auto it = t.rounds.find(key);
    if (it == t.rounds.end()) return false;
    out = it->second.route;
    return true;
}

void sumcheck_route_store(const RoundKey &key, const RoundRoute &route, double us) {
    TuningTable &t = table();
    std::lock_guard<std::mutex> lock(t.mu);
    load_env_locked(t);
    t.rounds[key] = RouteEntry{route, us};
}

}  // namespace hp

extern "C" HpCudaStatus hp_cuda_v1_msm_tuning_save(const char *path) {
    return guard([&] {
        require(path != nullptr);
        hp::TuningTable &t = hp::table();
        std::lock_guard<std::mutex> lock(t.mu);
        hp::load_env_locked(t);
        std::ofstream f(path, std::ios::trunc);
        require(bool(f));
        f << "hp_cuda msm tuning 1\n";
        f << "device " << t.device << "\n";
        char line[160];
        for (const auto &kv : t.alone) {
            std::snprintf(line, sizeof line, "alone %d %d %u %u %.4f\n", kv.first, kv.second.t.c, kv.second.t.seg,
                          kv.second.t.chunk, kv.second.ms);
            f << line;
        }
        for (const auto &kv : t.many) {
            std::snprintf(line, sizeof line, "many %d %u %.4f\n", kv.first, kv.second.chunk, kv.second.ms);
            f << line;
        }
        for (const auto &kv : t.rounds) {
            std::snprintf(line, sizeof line, "round %d %d %d %d %u %u %.2f\n", kv.first.log2_pairs,
                          kv.first.max_arity, kv.first.slots, kv.first.fold, unsigned(kv.second.route.kernel),
                          unsigned(kv.second.route.per_sm), kv.second.us);
            f << line;
        }
        f.flush();
        require(bool(f));
    });
}

extern "C" HpCudaStatus hp_cuda_v1_msm_tuning_load(const char *path, const char *device) {
    return guard([&] {
        require(path != nullptr);
        hp::Parsed parsed;
        if (!hp::parse_file(path, parsed)) fail(HP_CUDA_STATUS_INVALID_PARAMETERS);
        if (device && parsed.device != "any" && parsed.device != hp::device_token(device))
            fail(HP_CUDA_STATUS_INVALID_PARAMETERS);
        hp::TuningTable &t = hp::table();
        std::lock_guard<std::mutex> lock(t.mu);
        hp::load_env_locked(t);
        hp::merge_into(t, parsed);
    });
}

extern "C" HpCudaStatus hp_cuda_v1_msm_tuning_clear(void) {
    return guard([&] {
        hp::TuningTable &t = hp::table();
        std::lock_guard<std::mutex> lock(t.mu);
        t.alone.clear();
        t.many.clear();
        t.rounds.clear();
        t.device = "any";
        t.env_checked = true;  // a cleared table stays empty
    });
}
