/* hp_cuda.hpp -- C++ host-side mirror of the reference's backend traits over
 * the hp_cuda C ABI (header-only, C++17, no CUDA headers needed).
 *
 *   Mle, MleBackend         backend/src/multilinear_polynomial.rs:22-121
 *   MultilinearKzgBackend   backend/src/multilinear_kzg.rs:20-55
 *   SumCheckProver          backend/src/sum_check.rs:17-38
 *   VirtualPolynomial       backend/src/virtual_polynomial.rs:44-235
 *   BackendError            backend/src/errors.rs:16-21 (status mapping of
 *                           ascend910b3/status.rs:170-195: kind 1 ->
 *                           InvalidParameters, any other failure ->
 *                           InvalidState)
 *
 * Method names, argument meaning and error behaviour follow the traits, as
 * the reference's Ascend wrapper (the backend/src/ascend910b3 modules) maps them onto
 * its bridge; field elements travel as the bridge's canonical packets
 * (ascend910b3/encoding.rs: Fr = 32-byte little-endian, G1 = 97 bytes, tag
 * 0 finite / 1 infinity, then x and y little-endian 48 bytes each).  A
 * CudaBackend owns one device context; handles (Mle clones share storage,
 * prepared parameters, prover states) keep it alive and release their
 * device resources when the last reference drops.  Like the reference's
 * handles they are neither thread-safe nor meant to cross threads.
 */
#pragma once

#include <array>
#include <cstdint>
#include <cstring>
#include <memory>
#include <optional>
#include <stdexcept>
#include <string>
#include <unordered_map>
#include <utility>
#include <vector>

#include "hp_cuda.h"

namespace hp_cuda {

using Fr = std::array<uint8_t, 32>;  // canonical little-endian
using G1 = std::array<uint8_t, 97>;  // tag || x || y

class BackendError : public std::runtime_error {
public:
    enum class Kind { InvalidParameters, InvalidState };
    BackendError(Kind kind, const std::string &what, int32_t native_code = 0)
        : std::runtime_error(what), kind(kind), native_code(native_code) {}
    Kind kind;
    int32_t native_code;
};

inline BackendError invalid_parameters(const std::string &what) {
    return BackendError(BackendError::Kind::InvalidParameters, what);
}

inline void check(HpCudaStatus s, const char *call) {
    if (s.kind == HP_CUDA_STATUS_SUCCESS) return;
    throw BackendError(s.kind == HP_CUDA_STATUS_INVALID_PARAMETERS ? BackendError::Kind::InvalidParameters
                                                                    : BackendError::Kind::InvalidState,
                       std::string(call) + " failed (status kind " + std::to_string(s.kind) + ")", s.native_code);
}

/* ---- canonical Fr arithmetic on the host (VirtualPolynomial coefficients,
 *      test oracles): Montgomery form with R = 2^256 over 4 x 64-bit limbs */
namespace fr {
namespace detail {
constexpr uint64_t P[4] = {0xffffffff00000001ULL, 0x53bda402fffe5bfeULL, 0x3339d80809a1d805ULL,
                           0x73eda753299d7d48ULL};
constexpr uint64_t R2[4] = {0xc999e990f3f29c6dULL, 0x2b6cedcb87925c23ULL, 0x05d314967254398fULL,
                            0x0748d9d99f59ff11ULL};
constexpr uint64_t INV = 0xfffffffeffffffffULL;  // -p^-1 mod 2^64
__extension__ typedef unsigned __int128 u128;  // GCC / Clang (x86-64, aarch64)
struct L {
    uint64_t v[4];
};
inline bool geq_p(const uint64_t *a) {
    for (int i = 3; i >= 0; i--)
        if (a[i] != P[i]) return a[i] > P[i];
    return true;
}
inline void sub_p(uint64_t *a) {
    u128 borrow = 0;
    for (int i = 0; i < 4; i++) {
        const u128 d = u128(a[i]) - P[i] - borrow;
        a[i] = uint64_t(d);
        borrow = (d >> 64) & 1;
    }
}
inline L mont_mul(const L &a, const L &b) {
    uint64_t t[6] = {0, 0, 0, 0, 0, 0};
    for (int i = 0; i < 4; i++) {
        u128 c = 0;
        for (int j = 0; j < 4; j++) {
            c += u128(a.v[j]) * b.v[i] + t[j];
            t[j] = uint64_t(c);
            c >>= 64;
        }
        c += t[4];
        t[4] = uint64_t(c);
        t[5] = uint64_t(c >> 64);
        const uint64_t m = t[0] * INV;
        c = u128(m) * P[0] + t[0];
        c >>= 64;
        for (int j = 1; j < 4; j++) {
            c += u128(m) * P[j] + t[j];
            t[j - 1] = uint64_t(c);
            c >>= 64;
        }
        c += t[4];
        t[3] = uint64_t(c);
        t[4] = t[5] + uint64_t(c >> 64);
    }
    L r;
    std::memcpy(r.v, t, 32);
    if (t[4] || geq_p(r.v)) sub_p(r.v);
    return r;
}
inline L load(const Fr &a) {
    L r;
    std::memcpy(r.v, a.data(), 32);
    if (geq_p(r.v)) throw invalid_parameters("non-canonical field element");
    return r;
}
inline Fr store(const L &a) {
    Fr r;
    std::memcpy(r.data(), a.v, 32);
    return r;
}
}  // namespace detail

inline Fr from_u64(uint64_t x) {
    Fr r{};
    for (int i = 0; i < 8; i++) r[i] = uint8_t(x >> (8 * i));
    return r;
}
inline Fr zero() { return Fr{}; }
inline Fr one() { return from_u64(1); }
inline bool is_zero(const Fr &a) {
    for (uint8_t b : a)
        if (b) return false;
    return true;
}
inline Fr add(const Fr &a, const Fr &b) {
    detail::L x = detail::load(a), y = detail::load(b), r;
    detail::u128 c = 0;
    for (int i = 0; i < 4; i++) {
        c += detail::u128(x.v[i]) + y.v[i];
        r.v[i] = uint64_t(c);
        c >>= 64;
    }
    if (c || detail::geq_p(r.v)) detail::sub_p(r.v);
    return detail::store(r);
}
inline Fr neg(const Fr &a) {
    if (is_zero(a)) return a;
    detail::L x = detail::load(a), r;
    detail::u128 borrow = 0;
    for (int i = 0; i < 4; i++) {
        const detail::u128 d = detail::u128(detail::P[i]) - x.v[i] - borrow;
        r.v[i] = uint64_t(d);
        borrow = (d >> 64) & 1;
    }
    return detail::store(r);
}
inline Fr sub(const Fr &a, const Fr &b) { return add(a, neg(b)); }
// canonical a * b: mont(a) * mont(b) then out of Montgomery form
inline Fr mul(const Fr &a, const Fr &b) {
    detail::L r2, one{{1, 0, 0, 0}};
    std::memcpy(r2.v, detail::R2, 32);
    const detail::L am = detail::mont_mul(detail::load(a), r2);
    const detail::L bm = detail::mont_mul(detail::load(b), r2);
    return detail::store(detail::mont_mul(detail::mont_mul(am, bm), one));
}
inline Fr pow(const Fr &a, const uint64_t *e, int limbs) {
    Fr acc = one();
    for (int i = limbs - 1; i >= 0; i--)
        for (int bit = 63; bit >= 0; bit--) {
            acc = mul(acc, acc);
            if ((e[i] >> bit) & 1) acc = mul(acc, a);
        }
    return acc;
}
inline Fr inv(const Fr &a) {  // a^(p-2); a != 0
    uint64_t e[4] = {detail::P[0] - 2, detail::P[1], detail::P[2], detail::P[3]};
    return pow(a, e, 4);
}
}  // namespace fr

class CudaBackend;

namespace detail {
struct Context {
    HpCudaContext *raw = nullptr;
    explicit Context(int device) { check(hp_cuda_v1_context_create(device, &raw), "context_create"); }
    Context(const Context &) = delete;
    Context &operator=(const Context &) = delete;
    ~Context() {
        if (raw) hp_cuda_v1_context_destroy(raw);
    }
};
struct Buffer {  // one device table; retired when its last Mle clone drops
    std::shared_ptr<Context> ctx;
    HpCudaDeviceAddress addr = nullptr;
    Buffer(std::shared_ptr<Context> c, HpCudaDeviceAddress a) : ctx(std::move(c)), addr(a) {}
    Buffer(const Buffer &) = delete;
    Buffer &operator=(const Buffer &) = delete;
    ~Buffer() {
        if (addr) hp_cuda_v1_buffer_retire(ctx->raw, addr);
    }
};
struct Params {
    std::shared_ptr<Context> ctx;
    HpCudaMultilinearKzgPreparedProverParam *raw = nullptr;
    Params(std::shared_ptr<Context> c, HpCudaMultilinearKzgPreparedProverParam *r) : ctx(std::move(c)), raw(r) {}
    Params(const Params &) = delete;
    Params &operator=(const Params &) = delete;
    ~Params() {
        if (raw) hp_cuda_v1_multilinear_kzg_params_destroy(ctx->raw, raw);
    }
};
struct State {
    std::shared_ptr<Context> ctx;
    HpCudaSumCheckProverState *raw = nullptr;
    State(std::shared_ptr<Context> c, HpCudaSumCheckProverState *r) : ctx(std::move(c)), raw(r) {}
    State(const State &) = delete;
    State &operator=(const State &) = delete;
    ~State() {
        if (raw) hp_cuda_v1_sumcheck_prover_state_destroy(ctx->raw, raw);
    }
};
}  // namespace detail

/* Mle (multilinear_polynomial.rs:22-27): a copy shares the storage, id() is
 * stable and distinct per allocation. */
class Mle {
public:
    Mle() = default;
    size_t num_vars() const { return nv_; }
    uintptr_t id() const { return reinterpret_cast<uintptr_t>(buf_.get()); }
    HpCudaDeviceAddress address() const { return buf_ ? buf_->addr : nullptr; }

private:
    friend class CudaBackend;
    Mle(std::shared_ptr<detail::Buffer> b, size_t nv) : buf_(std::move(b)), nv_(nv) {}
    std::shared_ptr<detail::Buffer> buf_;
    size_t nv_ = 0;
};

struct VPAuxInfo {
    size_t max_degree = 0;
    size_t num_variables = 0;
};

/* VirtualPolynomial (virtual_polynomial.rs:44-235): sum of coefficient-
 * weighted products of shared MLE handles; flattened factors deduplicated
 * by handle identity in first-insertion order; a failing call leaves the
 * polynomial unchanged. */
class VirtualPolynomial {
public:
    explicit VirtualPolynomial(size_t num_variables) { aux_info.num_variables = num_variables; }
    static VirtualPolynomial new_from_mle(const Mle &mle, const Fr &coefficient) {
        VirtualPolynomial vp(mle.num_vars());
        vp.aux_info.max_degree = 1;
        vp.flattened_.push_back(mle);
        vp.lookup_[mle.id()] = 0;
        vp.products.push_back({fr::detail::store(fr::detail::load(coefficient)), {0}});
        return vp;
    }
    void add_mle_list(const std::vector<Mle> &mle_list, const Fr &coefficient) {
        if (mle_list.empty()) throw invalid_parameters("input mle_list is empty");
        for (const Mle &m : mle_list)
            if (m.num_vars() != aux_info.num_variables)
                throw invalid_parameters("product has a multiplicand with wrong number of variables");
        fr::detail::load(coefficient);  // canonical check before any change
        aux_info.max_degree = std::max(aux_info.max_degree, mle_list.size());
        std::vector<size_t> indexed;
        for (const Mle &m : mle_list) indexed.push_back(index_of(m));
        products.push_back({coefficient, std::move(indexed)});
    }
    void mul_by_mle(const Mle &mle, const Fr &coefficient) {
        if (mle.num_vars() != aux_info.num_variables)
            throw invalid_parameters("product has a multiplicand with wrong number of variables");
        fr::detail::load(coefficient);
        const size_t idx = index_of(mle);
        for (auto &p : products) {
            p.first = fr::mul(p.first, coefficient);
            p.second.push_back(idx);
        }
        aux_info.max_degree += 1;
    }
    const std::vector<Mle> &flattened_ml_extensions() const { return flattened_; }

    VPAuxInfo aux_info;
    std::vector<std::pair<Fr, std::vector<size_t>>> products;

private:
    size_t index_of(const Mle &m) {
        auto it = lookup_.find(m.id());
        if (it != lookup_.end()) return it->second;
        const size_t idx = flattened_.size();
        lookup_[m.id()] = idx;
        flattened_.push_back(m);
        return idx;
    }
    std::vector<Mle> flattened_;
    std::unordered_map<uintptr_t, size_t> lookup_;
};

class PreparedProverParam {
public:
    size_t num_vars() const { return nv_; }

private:
    friend class CudaBackend;
    PreparedProverParam(std::shared_ptr<detail::Params> p, size_t nv) : p_(std::move(p)), nv_(nv) {}
    std::shared_ptr<detail::Params> p_;
    size_t nv_ = 0;
};

class SumCheckProverState {
public:
    size_t max_degree() const { return degree_; }
    size_t factor_count() const { return factors_; }

private:
    friend class CudaBackend;
    SumCheckProverState(std::shared_ptr<detail::State> s, size_t d, size_t f) : s_(std::move(s)), degree_(d),
                                                                              factors_(f) {}
    std::shared_ptr<detail::State> s_;
    size_t degree_ = 0, factors_ = 0;
};

/* MleBackend + MultilinearKzgBackend + SumCheckProver over one GB300 context. */
class CudaBackend {
public:
    explicit CudaBackend(int device = 0) : ctx_(std::make_shared<detail::Context>(device)) {}
    HpCudaContext *raw() const { return ctx_->raw; }

    /* ---- MleBackend (multilinear_polynomial.rs:33-121) ---- */
    Mle mle_from_evaluations(size_t num_vars, const std::vector<Fr> &evaluations) const {
        if (num_vars >= 64 || evaluations.size() != (size_t(1) << num_vars))
            throw invalid_parameters("evaluation count does not match the number of variables");
        HpCudaDeviceAddress out = nullptr;
        check(hp_cuda_v1_mle_upload(ctx_->raw, num_vars, evaluations.data()->data(), evaluations.size(), &out),
              "mle_upload");
        return wrap(out, num_vars);
    }
    std::vector<Fr> download(const Mle &m) const {  // canonical table (parity checks)
        own(m);
        std::vector<Fr> out(size_t(1) << m.num_vars());
        check(hp_cuda_v1_mle_download(ctx_->raw, m.address(), m.num_vars(), out.data()->data(), out.size()),
              "mle_download");
        return out;
    }
    Mle linear_combination(const std::vector<Mle> &polynomials, const std::vector<Fr> &coefficients) const {
        if (polynomials.empty()) throw invalid_parameters("linear combination requires nonempty polynomials");
        const size_t nv = polynomials[0].num_vars();
        if (polynomials.size() != coefficients.size()) throw invalid_parameters("coefficient count mismatch");
        for (const Mle &p : polynomials) {
            own(p);
            if (p.num_vars() != nv) throw invalid_parameters("linear combination requires matching dimensions");
        }
        const auto addrs = addresses(polynomials);
        HpCudaDeviceAddress out = nullptr;
        check(hp_cuda_v1_mle_linear_combination(ctx_->raw, nv, addrs.data(), coefficients.data()->data(),
                                                polynomials.size(), &out),
              "mle_linear_combination");
        return wrap(out, nv);
    }
    Fr evaluate(const Mle &polynomial, const std::vector<Fr> &point) const {
        own(polynomial);
        if (point.size() != polynomial.num_vars()) throw invalid_parameters("wrong number of variables");
        Fr out{};
        check(hp_cuda_v1_mle_evaluate(ctx_->raw, polynomial.address(), polynomial.num_vars(),
                                      point.empty() ? nullptr : point.data()->data(), out.data()),
              "mle_evaluate");
        return out;
    }
    Mle build_eq_x_r(const std::vector<Fr> &r) const {
        if (r.empty()) throw invalid_parameters("r length is 0");
        HpCudaDeviceAddress out = nullptr;
        check(hp_cuda_v1_mle_build_eq_x_r(ctx_->raw, r.data()->data(), r.size(), &out), "mle_build_eq_x_r");
        return wrap(out, r.size());
    }
    Mle compute_frac_poly(const std::vector<Mle> &fxs, const std::vector<Mle> &gxs) const {
        if (fxs.empty() || fxs.size() != gxs.size()) throw invalid_parameters("frac requires equal nonempty lists");
        const size_t nv = fxs[0].num_vars();
        for (const auto *list : {&fxs, &gxs})
            for (const Mle &p : *list) {
                own(p);
                if (p.num_vars() != nv) throw invalid_parameters("frac requires matching dimensions");
            }
        const auto f = addresses(fxs), g = addresses(gxs);
        HpCudaDeviceAddress out = nullptr;
        check(hp_cuda_v1_mle_compute_frac_poly(ctx_->raw, nv, f.data(), g.data(), fxs.size(), &out),
              "mle_compute_frac_poly");
        return wrap(out, nv);
    }
    Mle compute_product_poly(const Mle &frac) const {
        own(frac);
        if (frac.num_vars() == 0) throw invalid_parameters("product polynomial requires at least one variable");
        HpCudaDeviceAddress out = nullptr;
        check(hp_cuda_v1_mle_compute_product_poly(ctx_->raw, frac.address(), frac.num_vars(), &out),
              "mle_compute_product_poly");
        return wrap(out, frac.num_vars());
    }
    std::pair<std::vector<Mle>, std::vector<Mle>> compute_nums_and_denoms(const Fr &beta, const Fr &gamma,
                                                                         const std::vector<Mle> &fxs,
                                                                         const std::vector<Mle> &gxs,
                                                                         const std::vector<Mle> &perms) const {
        const size_t k = fxs.size();
        if (k == 0 || gxs.size() != k || perms.size() != k)
            throw invalid_parameters("nums/denoms require equal nonempty lists");
        const size_t nv = fxs[0].num_vars();
        for (const auto *list : {&fxs, &gxs, &perms})
            for (const Mle &p : *list) {
                own(p);
                if (p.num_vars() != nv) throw invalid_parameters("nums/denoms require matching dimensions");
            }
        const auto f = addresses(fxs), g = addresses(gxs), s = addresses(perms);
        std::vector<HpCudaDeviceAddress> nums(k, nullptr), dens(k, nullptr);
        check(hp_cuda_v1_mle_compute_nums_and_denoms(ctx_->raw, nv, beta.data(), gamma.data(), f.data(), g.data(),
                                                     s.data(), k, nums.data(), dens.data()),
              "mle_compute_nums_and_denoms");
        std::pair<std::vector<Mle>, std::vector<Mle>> out;
        for (size_t i = 0; i < k; i++) {
            out.first.push_back(wrap(nums[i], nv));
            out.second.push_back(wrap(dens[i], nv));
        }
        return out;
    }
    std::pair<Mle, Mle> compute_product_factors(const Mle &frac, const Mle &prod) const {
        own(frac);
        own(prod);
        const size_t nv = frac.num_vars();
        if (nv == 0) throw invalid_parameters("product factors require at least one variable");
        if (prod.num_vars() != nv) throw invalid_parameters("product factor inputs have different variable counts");
        HpCudaDeviceAddress a = nullptr, b = nullptr;
        check(hp_cuda_v1_mle_compute_product_factors(ctx_->raw, frac.address(), prod.address(), nv, &a, &b),
              "mle_compute_product_factors");
        Mle p1 = wrap(a, nv);
        return {p1, wrap(b, nv)};
    }

    /* ---- MultilinearKzgBackend (multilinear_kzg.rs:20-55) ---- */
    PreparedProverParam prepare_prover_param(size_t num_vars, const std::vector<std::vector<G1>> &powers_of_g) const {
        if (powers_of_g.size() != num_vars + 1) throw invalid_parameters("SRS must contain num_vars + 1 layers");
        HpCudaMultilinearKzgPreparedProverParam *raw = nullptr;
        check(hp_cuda_v1_multilinear_kzg_params_create(ctx_->raw, num_vars, &raw), "multilinear_kzg_params_create");
        auto p = std::make_shared<detail::Params>(ctx_, raw);
        for (size_t i = 0; i <= num_vars; i++) {
            const size_t count = i < num_vars ? size_t(1) << (num_vars - i) : 1;
            if (powers_of_g[i].size() != count) throw invalid_parameters("SRS layer has an incorrect point count");
            check(hp_cuda_v1_multilinear_kzg_params_upload_layer(ctx_->raw, raw, i, powers_of_g[i].data()->data(),
                                                                 count),
                  "multilinear_kzg_params_upload_layer");
        }
        return PreparedProverParam(p, num_vars);
    }
    G1 commit(const PreparedProverParam &pp, const Mle &polynomial) const {
        own(pp);
        own(polynomial);
        G1 out{};
        check(hp_cuda_v1_multilinear_kzg_commit(ctx_->raw, pp.p_->raw, polynomial.address(), polynomial.num_vars(),
                                                out.data()),
              "multilinear_kzg_commit");
        return out;
    }
    std::vector<G1> multi_commit(const PreparedProverParam &pp, const std::vector<Mle> &polynomials) const {
        own(pp);
        if (polynomials.empty()) return {};
        std::vector<size_t> nvs;
        for (const Mle &p : polynomials) {
            own(p);
            nvs.push_back(p.num_vars());
        }
        const auto addrs = addresses(polynomials);
        std::vector<G1> out(polynomials.size());
        check(hp_cuda_v1_multilinear_kzg_multi_commit(ctx_->raw, pp.p_->raw, addrs.data(), nvs.data(),
                                                      polynomials.size(), out.data()->data()),
              "multilinear_kzg_multi_commit");
        return out;
    }
    std::pair<std::vector<G1>, Fr> open(const PreparedProverParam &pp, const Mle &polynomial,
                                        const std::vector<Fr> &point) const {
        own(pp);
        own(polynomial);
        const size_t nv = polynomial.num_vars();
        if (point.size() != nv) throw invalid_parameters("polynomial num_vars does not match point length");
        std::vector<G1> q(std::max<size_t>(nv, 1));
        Fr ev{};
        check(hp_cuda_v1_multilinear_kzg_open(ctx_->raw, pp.p_->raw, polynomial.address(), nv,
                                              point.empty() ? nullptr : point.data()->data(), q.data()->data(),
                                              ev.data()),
              "multilinear_kzg_open");
        q.resize(nv);
        return {q, ev};
    }

    /* ---- SumCheckProver (sum_check.rs:17-38), product encoding of
     *      ascend910b3/sum_check.rs:32-90 ---- */
    SumCheckProverState prover_init(const VirtualPolynomial &vp) const {
        const size_t nv = vp.aux_info.num_variables, d = vp.aux_info.max_degree;
        if (nv == 0 || d == 0) throw invalid_parameters("SumCheck requires positive variable count and degree");
        const auto &factors = vp.flattened_ml_extensions();
        for (const Mle &f : factors) {
            own(f);
            if (f.num_vars() != nv) throw invalid_parameters("SumCheck factor dimensions do not match");
        }
        std::vector<size_t> offsets{0}, indices;
        std::vector<Fr> coefs;
        for (const auto &p : vp.products) {
            if (p.second.empty() || p.second.size() > d)
                throw invalid_parameters("SumCheck product must have between one and max_degree multiplicands");
            for (size_t i : p.second) {
                if (i >= factors.size()) throw invalid_parameters("SumCheck product references an unknown factor");
                indices.push_back(i);
            }
            offsets.push_back(indices.size());
            coefs.push_back(p.first);
        }
        const auto addrs = addresses(factors);
        HpCudaSumCheckProverState *raw = nullptr;
        check(hp_cuda_v1_sumcheck_prover_state_create(
                  ctx_->raw, nv, d, addrs.empty() ? nullptr : addrs.data(), addrs.size(),
                  coefs.empty() ? nullptr : coefs.data()->data(), offsets.data(), coefs.size(),
                  indices.empty() ? nullptr : indices.data(), indices.size(), &raw),
              "sumcheck_prover_state_create");
        return SumCheckProverState(std::make_shared<detail::State>(ctx_, raw), d, factors.size());
    }
    std::vector<Fr> prove_round_and_update_state(SumCheckProverState &state,
                                                 const std::optional<Fr> &challenge) const {
        own(state);
        std::vector<Fr> out(state.max_degree() + 1);
        check(hp_cuda_v1_sumcheck_prover_state_round(ctx_->raw, state.s_->raw,
                                                     challenge ? challenge->data() : nullptr, out.data()->data(),
                                                     out.size()),
              "sumcheck_prover_state_round");
        return out;
    }
    /* beyond the trait: the factors' values at the last challenge */
    std::vector<Fr> final_evaluations(SumCheckProverState &state, const Fr &challenge) const {
        own(state);
        std::vector<Fr> out(std::max<size_t>(state.factor_count(), 1));
        check(hp_cuda_v1_sumcheck_prover_state_final_evaluations(ctx_->raw, state.s_->raw, challenge.data(),
                                                                 out.data()->data(), state.factor_count()),
              "sumcheck_prover_state_final_evaluations");
        out.resize(state.factor_count());
        return out;
    }

    /* ---- MSM autotuner (no counterpart in the reference; see hp_cuda.h) ----
     * mode 0: one entry per size, and pp's layers are re-prepared with them;
     * mode 1: one entry for a launch shared by all the sizes (<= 64). */
    std::vector<HpCudaMsmTuning> msm_autotune(const PreparedProverParam &pp, const std::vector<size_t> &num_vars,
                                              int mode = 0) const {
        own(pp);
        if (num_vars.empty()) return {};
        std::vector<HpCudaMsmTuning> out(mode == 0 ? num_vars.size() : 1);
        check(hp_cuda_v1_msm_autotune(ctx_->raw, pp.p_->raw, num_vars.data(), num_vars.size(), mode, out.data()),
              "msm_autotune");
        return out;
    }

private:
    Mle wrap(HpCudaDeviceAddress a, size_t nv) const { return Mle(std::make_shared<detail::Buffer>(ctx_, a), nv); }
    void own(const Mle &m) const {
        if (!m.buf_ || m.buf_->ctx != ctx_) throw invalid_parameters("MLE handle belongs to another backend");
    }
    void own(const PreparedProverParam &pp) const {
        if (!pp.p_ || pp.p_->ctx != ctx_) throw invalid_parameters("prover parameters belong to another backend");
    }
    void own(const SumCheckProverState &st) const {
        if (!st.s_ || st.s_->ctx != ctx_) throw invalid_parameters("prover state belongs to another backend");
    }
    static std::vector<HpCudaDeviceAddress> addresses(const std::vector<Mle> &ms) {
        std::vector<HpCudaDeviceAddress> a;
        a.reserve(ms.size());
        for (const Mle &m : ms) a.push_back(m.address());
        return a;
    }
    std::shared_ptr<detail::Context> ctx_;
};

/* The process-wide MSM tuning table (hp_cuda_v1_msm_tuning_*). */
namespace tuning {
struct Geometry {
    uint32_t window_bits, segment, chunk;
};
/* mode 0: the geometry a new layer of `size` points takes; mode 1: the chunk
 * (window_bits = segment = 0) of a shared launch of `size` records. */
inline Geometry query(int mode, size_t size) {
    uint32_t g[3] = {0, 0, 0};
    check(hp_cuda_v1_msm_tuning_query(mode, size, g), "msm_tuning_query");
    return Geometry{g[0], g[1], g[2]};
}
inline void save(const std::string &path) { check(hp_cuda_v1_msm_tuning_save(path.c_str()), "msm_tuning_save"); }
/* device: reject a file measured on another device name; empty: accept any. */
inline void load(const std::string &path, const std::string &device = std::string()) {
    check(hp_cuda_v1_msm_tuning_load(path.c_str(), device.empty() ? nullptr : device.c_str()), "msm_tuning_load");
}
inline void clear() { check(hp_cuda_v1_msm_tuning_clear(), "msm_tuning_clear"); }
}  // namespace tuning

}  // namespace hp_cuda
