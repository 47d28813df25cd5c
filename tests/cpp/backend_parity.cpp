// backend_parity.cpp -- the reference's device-backend integration tests
// (backend/src/ascend910b3/integration_tests.rs), restated in C++ against the
// GB300 backend through include/hp_cuda.hpp, with the oracle library
// (oracle/hp_oracle.h, the C restatement of the reference's CpuBackend) as the
// CPU side.  Test names follow the reference's; each checks the same
// properties: device result == CPU result == directly computed expectation,
// evaluations at boolean and random points, inputs left unchanged, and the
// error contract (InvalidParameters / InvalidState).  Exit status 0 when every
// check passes.  Needs a GPU.
#include <cstdio>
#include <cstdlib>
#include <functional>
#include <string>
#include <vector>

#include "hp_cuda.hpp"
#include "hp_oracle.h"

using namespace hp_cuda;
using Table = std::vector<Fr>;

static int g_checks = 0, g_failures = 0;

#define CHECK(cond)                                                                      \
    do {                                                                                 \
        g_checks++;                                                                      \
        if (!(cond)) {                                                                   \
            g_failures++;                                                                \
            std::fprintf(stderr, "  %s:%d: CHECK failed: %s\n", __FILE__, __LINE__, #cond); \
        }                                                                                \
    } while (0)

template <class F>
static void expect_error(BackendError::Kind kind, F f, const char *what) {
    g_checks++;
    try {
        f();
    } catch (const BackendError &e) {
        if (e.kind == kind) return;
        g_failures++;
        std::fprintf(stderr, "  %s: wrong error kind (%s)\n", what, e.what());
        return;
    }
    g_failures++;
    std::fprintf(stderr, "  %s: no error\n", what);
}
#define EXPECT_INVALID_PARAMETERS(expr) \
    expect_error(BackendError::Kind::InvalidParameters, [&] { (void)(expr); }, #expr)
#define EXPECT_INVALID_STATE(expr) expect_error(BackendError::Kind::InvalidState, [&] { (void)(expr); }, #expr)

// ---------------------------------------------------------------------------
// fixtures (seeded ChaCha20 Fr streams of the oracle)
// ---------------------------------------------------------------------------

static Table field_table(size_t nv, uint64_t seed) {
    Table t(size_t(1) << nv);
    or_random_fr(seed, 0, t.size(), t.data()->data());
    return t;
}

static Table nonzero_table(size_t nv, uint64_t seed) {
    Table t = field_table(nv, seed);
    for (Fr &v : t)
        if (fr::is_zero(v)) v = fr::one();
    return t;
}

static Fr fr_of(uint64_t seed, uint64_t index) {
    Fr r;
    or_random_fr(seed, index, 1, r.data());
    return r;
}

static std::vector<Fr> boolean_point(size_t nv, size_t index) {
    std::vector<Fr> p(nv);
    for (size_t i = 0; i < nv; i++) p[i] = ((index >> i) & 1) ? fr::one() : fr::zero();
    return p;
}

// boolean corners plus random points
static std::vector<std::vector<Fr>> comparison_points(size_t nv, uint64_t seed) {
    std::vector<std::vector<Fr>> pts;
    pts.push_back(boolean_point(nv, 0));
    if (nv > 0) pts.push_back(boolean_point(nv, (size_t(1) << nv) - 1));
    for (uint64_t k = 0; k < 3; k++) {
        std::vector<Fr> p(nv);
        for (size_t i = 0; i < nv; i++) p[i] = fr_of(seed, 16 * k + i);
        pts.push_back(p);
    }
    return pts;
}

// the multilinear extension of `table` at `point` (point[0] <-> bit 0)
static Fr multilinear_eval(Table f, const std::vector<Fr> &point) {
    for (const Fr &r : point) {
        Table g(f.size() / 2);
        for (size_t b = 0; b < g.size(); b++) g[b] = fr::add(f[2 * b], fr::mul(r, fr::sub(f[2 * b + 1], f[2 * b])));
        f.swap(g);
    }
    return f[0];
}

static std::vector<const uint8_t *> ptrs(const std::vector<Table> &ts) {
    std::vector<const uint8_t *> p;
    for (const Table &t : ts) p.push_back(t.data()->data());
    return p;
}

static std::vector<Mle> upload_all(const CudaBackend &be, size_t nv, const std::vector<Table> &ts) {
    std::vector<Mle> m;
    for (const Table &t : ts) m.push_back(be.mle_from_evaluations(nv, t));
    return m;
}

// device handle == expected table == CPU table, and evaluations agree
static void assert_mle_matches(const CudaBackend &be, const Mle &device, const Table &cpu, const Table &expected,
                               const std::vector<std::vector<Fr>> &points) {
    CHECK(device.num_vars() < 64 && (size_t(1) << device.num_vars()) == expected.size());
    CHECK(be.download(device) == expected);
    CHECK(cpu == expected);
    for (const auto &pt : points) {
        const Fr want = multilinear_eval(expected, pt);
        CHECK(be.evaluate(device, pt) == want);
        Fr got{};
        CHECK(or_mle_evaluate(cpu.data()->data(), device.num_vars(), pt.empty() ? nullptr : pt.data()->data(),
                              got.data()) == 0 &&
              got == want);
    }
}

// ---------------------------------------------------------------------------
// G1 packets: bridge form (97 bytes, tag + x + y) <-> oracle affine (96 bytes)
// ---------------------------------------------------------------------------

static G1 packet_of(const uint8_t *affine96) {
    G1 p{};
    bool zero = true;
    for (int i = 0; i < 96; i++) zero = zero && affine96[i] == 0;
    p[0] = zero ? 1 : 0;
    if (!zero) std::memcpy(p.data() + 1, affine96, 96);
    return p;
}

// testing SRS of `nv` variables (seed): nv + 1 layers of 2^(nv-i) packets
static void fixture_failed(const char *what) { throw std::runtime_error(std::string("fixture failed: ") + what); }

static std::vector<std::vector<G1>> srs_layers(size_t nv, uint64_t seed, std::vector<std::vector<uint8_t>> *affine) {
    // the oracle's generator starts at one variable: nv = 0 is the last layer
    // [g] of the one-variable parameters
    const size_t gen_nv = nv == 0 ? 1 : nv;
    const size_t total = (size_t(1) << (gen_nv + 1)) - 1;
    std::vector<uint8_t> raw(96 * total);
    if (or_srs_gen(gen_nv, seed, raw.data()) != 0) fixture_failed("or_srs_gen");
    std::vector<std::vector<G1>> layers;
    size_t off = nv == 0 ? total - 1 : 0;
    for (size_t i = 0; i <= nv; i++) {
        const size_t count = i < nv ? size_t(1) << (nv - i) : 1;
        std::vector<G1> layer;
        for (size_t k = 0; k < count; k++) layer.push_back(packet_of(raw.data() + 96 * (off + k)));
        if (affine) affine->emplace_back(raw.begin() + 96 * off, raw.begin() + 96 * (off + count));
        layers.push_back(layer);
        off += count;
    }
    return layers;
}

// ---------------------------------------------------------------------------
// MLE operations
// ---------------------------------------------------------------------------

static void linear_combination_and_evaluate_match_cpu_for_all_dimensions(const CudaBackend &be) {
    for (size_t nv = 0; nv <= 8; nv++) {
        const std::vector<Table> inputs = {field_table(nv, 0xA11CE), field_table(nv, 0xB0B), field_table(nv, 0xC0FFEE)};
        const std::vector<Fr> coefs = {fr::zero(), fr::neg(fr::one()), fr::from_u64(0xDEADBEEFull)};
        Table expected(size_t(1) << nv, fr::zero());
        for (size_t j = 0; j < 3; j++)
            for (size_t i = 0; i < expected.size(); i++) expected[i] = fr::add(expected[i], fr::mul(coefs[j], inputs[j][i]));
        const auto handles = upload_all(be, nv, inputs);
        Table cpu(expected.size());
        const auto p = ptrs(inputs);
        CHECK(or_mle_linear_combination(nv, p.data(), coefs.data()->data(), 3, cpu.data()->data()) == 0);
        const Mle got = be.linear_combination(handles, coefs);
        assert_mle_matches(be, got, cpu, expected, comparison_points(nv, 0x51));
        // a zero combination keeps the variable count
        const Mle zero = be.linear_combination(handles, {fr::zero(), fr::zero(), fr::zero()});
        CHECK(zero.num_vars() == nv);
        CHECK(be.evaluate(zero, comparison_points(nv, 0x52)[0]) == fr::zero());
        // inputs are left unchanged
        for (size_t j = 0; j < 3; j++) CHECK(be.download(handles[j]) == inputs[j]);
    }
    const Mle one = be.mle_from_evaluations(1, field_table(1, 1));
    const Mle two = be.mle_from_evaluations(2, field_table(2, 2));
    EXPECT_INVALID_PARAMETERS(be.linear_combination({one}, {}));
    EXPECT_INVALID_PARAMETERS(be.linear_combination({one, two}, {fr::one(), fr::one()}));
    EXPECT_INVALID_PARAMETERS(be.linear_combination({}, {}));
    EXPECT_INVALID_PARAMETERS(be.evaluate(one, {}));
}

static void eq_polynomial_matches_closed_form_and_cpu(const CudaBackend &be) {
    for (size_t nv = 1; nv <= 8; nv++) {
        std::vector<Fr> r(nv);
        for (size_t i = 0; i < nv; i++) r[i] = fr_of(0xE9 ^ nv, i);
        r[0] = fr::zero();
        r[nv - 1] = fr::neg(fr::one());
        Table expected(size_t(1) << nv);
        for (size_t x = 0; x < expected.size(); x++) {
            Fr v = fr::one();
            for (size_t b = 0; b < nv; b++) v = fr::mul(v, ((x >> b) & 1) ? r[b] : fr::sub(fr::one(), r[b]));
            expected[x] = v;
        }
        Table cpu(expected.size());
        CHECK(or_mle_build_eq_x_r(r.data()->data(), nv, cpu.data()->data()) == 0);
        assert_mle_matches(be, be.build_eq_x_r(r), cpu, expected, comparison_points(nv, 0xEA));
    }
    EXPECT_INVALID_PARAMETERS(be.build_eq_x_r({}));
}

static Table frac_expected(const std::vector<Table> &nums, const std::vector<Table> &dens) {
    Table e(nums[0].size());
    for (size_t i = 0; i < e.size(); i++) {
        Fr n = fr::one(), d = fr::one();
        for (const Table &t : nums) n = fr::mul(n, t[i]);
        for (const Table &t : dens) d = fr::mul(d, t[i]);
        e[i] = fr::mul(n, fr::inv(d));
    }
    return e;
}

static void fraction_polynomial_matches_cpu_and_rejects_zero_denominators(const CudaBackend &be) {
    for (size_t nv = 0; nv <= 8; nv++) {
        const std::vector<Table> nums = {field_table(nv, 0xF1), field_table(nv, 0xF2), field_table(nv, 0xF3)};
        const std::vector<Table> dens = {nonzero_table(nv, 0xD1), nonzero_table(nv, 0xD2), nonzero_table(nv, 0xD3)};
        const Table expected = frac_expected(nums, dens);
        Table cpu(expected.size());
        const auto pn = ptrs(nums), pd = ptrs(dens);
        CHECK(or_mle_frac(nv, pn.data(), pd.data(), 3, cpu.data()->data()) == 0);
        const auto hn = upload_all(be, nv, nums), hd = upload_all(be, nv, dens);
        assert_mle_matches(be, be.compute_frac_poly(hn, hd), cpu, expected, comparison_points(nv, 0xF4));
        CHECK(be.download(hn[0]) == nums[0]);
    }
    for (size_t nv = 0; nv <= 3; nv++) {
        const size_t n = size_t(1) << nv;
        const Table num = field_table(nv, 0xCC);
        Table den = nonzero_table(nv, 0xDD);
        for (size_t pos : {size_t(0), n - 1}) {
            den[pos] = fr::zero();
            EXPECT_INVALID_PARAMETERS(be.compute_frac_poly({be.mle_from_evaluations(nv, num)},
                                                           {be.mle_from_evaluations(nv, den)}));  // x / 0
            Table zn = num;
            zn[pos] = fr::zero();
            EXPECT_INVALID_PARAMETERS(be.compute_frac_poly({be.mle_from_evaluations(nv, zn)},
                                                           {be.mle_from_evaluations(nv, den)}));  // 0 / 0
            den[pos] = fr::one();
        }
        // a zero made only by the product of the denominator factors
        Table f1 = nonzero_table(nv, 0xD4);
        f1[0] = fr::zero();
        EXPECT_INVALID_PARAMETERS(be.compute_frac_poly(
            {be.mle_from_evaluations(nv, num)},
            {be.mle_from_evaluations(nv, f1), be.mle_from_evaluations(nv, nonzero_table(nv, 0xD5))}));
    }
    const Mle h = be.mle_from_evaluations(2, field_table(2, 7));
    EXPECT_INVALID_PARAMETERS(be.compute_frac_poly({h}, {}));
    EXPECT_INVALID_PARAMETERS(be.compute_frac_poly({h}, {h, h}));
    EXPECT_INVALID_PARAMETERS(be.compute_frac_poly({}, {}));
}

static void fraction_zero_detection_spans_grid_stride_tiles_without_poisoning(const CudaBackend &be) {
    const size_t nv = 12, n = size_t(1) << nv;
    Table num = nonzero_table(nv, 0xF0);
    const Table den = nonzero_table(nv, 0xF1);
    const Mle hn = be.mle_from_evaluations(nv, num);
    for (size_t pos : {size_t(0), n - 1, n / 2 + 7}) {
        Table z = den;
        z[pos] = fr::zero();
        EXPECT_INVALID_PARAMETERS(be.compute_frac_poly({hn}, {be.mle_from_evaluations(nv, z)}));
        Table zn = num;
        zn[pos] = fr::zero();
        EXPECT_INVALID_PARAMETERS(be.compute_frac_poly({be.mle_from_evaluations(nv, zn)}, {be.mle_from_evaluations(nv, z)}));
    }
    // the failed calls poison nothing: the same inputs then divide correctly
    const Mle hd = be.mle_from_evaluations(nv, den);
    Table cpu(n);
    const uint8_t *pn = num.data()->data(), *pd = den.data()->data();
    CHECK(or_mle_frac(nv, &pn, &pd, 1, cpu.data()->data()) == 0);
    assert_mle_matches(be, be.compute_frac_poly({hn}, {hd}), cpu, frac_expected({num}, {den}),
                       comparison_points(nv, 0xF6));
}

static void product_recurrence_and_factors_match_cpu(const CudaBackend &be) {
    for (size_t nv = 1; nv <= 10; nv++) {
        const size_t n = size_t(1) << nv;
        const Table frac = nonzero_table(nv, 0x9A0 + nv);
        // prod[0..n/2) = frac[2i] frac[2i+1]; prod[n/2 + j] = prod[2j] prod[2j+1]; prod[n-1] = 0
        Table prod(n, fr::zero());
        for (size_t i = 0; i < n / 2; i++) prod[i] = fr::mul(frac[2 * i], frac[2 * i + 1]);
        for (size_t j = 0; n / 2 + j < n - 1; j++) prod[n / 2 + j] = fr::mul(prod[2 * j], prod[2 * j + 1]);
        Table cpu(n);
        CHECK(or_mle_product_poly(frac.data()->data(), nv, cpu.data()->data()) == 0);
        const Mle hf = be.mle_from_evaluations(nv, frac);
        const Mle hp = be.compute_product_poly(hf);
        assert_mle_matches(be, hp, cpu, prod, comparison_points(nv, 0x9B));
        // p1 = even entries of (frac || prod), p2 = odd entries
        Table p1(n), p2(n);
        for (size_t i = 0; i < n / 2; i++) {
            p1[i] = frac[2 * i];
            p2[i] = frac[2 * i + 1];
            p1[n / 2 + i] = prod[2 * i];
            p2[n / 2 + i] = prod[2 * i + 1];
        }
        Table c1(n), c2(n);
        CHECK(or_mle_product_factors(frac.data()->data(), prod.data()->data(), nv, c1.data()->data(),
                                     c2.data()->data()) == 0);
        const auto f = be.compute_product_factors(hf, hp);
        assert_mle_matches(be, f.first, c1, p1, comparison_points(nv, 0x9C));
        assert_mle_matches(be, f.second, c2, p2, comparison_points(nv, 0x9D));
    }
    const Mle scalar = be.mle_from_evaluations(0, {fr::one()});
    EXPECT_INVALID_PARAMETERS(be.compute_product_poly(scalar));
    EXPECT_INVALID_PARAMETERS(be.compute_product_factors(be.mle_from_evaluations(2, field_table(2, 1)),
                                                         be.mle_from_evaluations(3, field_table(3, 1))));
}

static void nums_and_denoms_match_cpu_with_nonidentity_permutations(const CudaBackend &be) {
    for (size_t nv = 1; nv <= 8; nv++) {
        const size_t n = size_t(1) << nv, k = 3;
        std::vector<Table> fxs, gxs, perms;
        for (size_t c = 0; c < k; c++) {
            fxs.push_back(field_table(nv, 0x5A0 + c));
            gxs.push_back(field_table(nv, 0x5B0 + c));
            // a permutation of the labels col * n + row: rotate rows, then columns
            Table p(n);
            for (size_t row = 0; row < n; row++) p[row] = fr::from_u64(((c + 1) % k) * n + (row * 5 + 3) % n);
            perms.push_back(p);
        }
        const Fr beta = fr_of(0x5C, nv), gamma = fr_of(0x5D, nv);
        std::vector<Table> en(k, Table(n)), ed(k, Table(n));
        for (size_t c = 0; c < k; c++)
            for (size_t row = 0; row < n; row++) {
                en[c][row] = fr::add(fr::add(fxs[c][row], fr::mul(beta, fr::from_u64(c * n + row))), gamma);
                ed[c][row] = fr::add(fr::add(gxs[c][row], fr::mul(beta, perms[c][row])), gamma);
            }
        std::vector<Table> cn(k, Table(n)), cd(k, Table(n));
        std::vector<uint8_t *> pcn, pcd;
        for (size_t c = 0; c < k; c++) {
            pcn.push_back(cn[c].data()->data());
            pcd.push_back(cd[c].data()->data());
        }
        const auto pf = ptrs(fxs), pg = ptrs(gxs), pp = ptrs(perms);
        CHECK(or_mle_nums_denoms(nv, beta.data(), gamma.data(), pf.data(), pg.data(), pp.data(), k, pcn.data(),
                                 pcd.data()) == 0);
        const auto got = be.compute_nums_and_denoms(beta, gamma, upload_all(be, nv, fxs), upload_all(be, nv, gxs),
                                                    upload_all(be, nv, perms));
        for (size_t c = 0; c < k; c++) {
            assert_mle_matches(be, got.first[c], cn[c], en[c], comparison_points(nv, 0x5E + c));
            assert_mle_matches(be, got.second[c], cd[c], ed[c], comparison_points(nv, 0x5F + c));
        }
    }
    const Mle a = be.mle_from_evaluations(2, field_table(2, 3));
    EXPECT_INVALID_PARAMETERS(be.compute_nums_and_denoms(fr::one(), fr::one(), {a}, {a}, {}));
    EXPECT_INVALID_PARAMETERS(be.compute_nums_and_denoms(fr::one(), fr::one(), {}, {}, {}));
}

// ---------------------------------------------------------------------------
// multilinear KZG
// ---------------------------------------------------------------------------

// sum_i values[i] * layer(param_vars - num_vars)[i], by the oracle's MSM
static G1 independent_commitment(const std::vector<std::vector<uint8_t>> &affine, size_t param_vars, size_t num_vars,
                                 const Table &values) {
    uint8_t out[96];
    if (or_msm(affine[param_vars - num_vars].data(), values.data()->data(), values.size(), out) != 0)
        fixture_failed("or_msm");
    return packet_of(out);
}

static std::pair<std::vector<G1>, Fr> cpu_open(const std::vector<std::vector<uint8_t>> &affine, size_t param_vars,
                                               const Table &values, size_t nv, const std::vector<Fr> &point) {
    std::vector<const uint8_t *> layers;
    for (size_t i = 0; i < nv; i++) layers.push_back(affine[param_vars - nv + 1 + i].data());
    std::vector<uint8_t> q(96 * std::max<size_t>(nv, 1));
    Fr ev{};
    if (or_kzg_open(layers.data(), values.data()->data(), nv, point.empty() ? nullptr : point.data()->data(), q.data(),
                    ev.data()) != 0)
        fixture_failed("or_kzg_open");
    std::vector<G1> proofs;
    for (size_t i = 0; i < nv; i++) proofs.push_back(packet_of(q.data() + 96 * i));
    return {proofs, ev};
}

static void commit_matches_cpu_and_independent_msm(const CudaBackend &be) {
    for (size_t pv : {size_t(0), size_t(1), size_t(2), size_t(4)}) {
        std::vector<std::vector<uint8_t>> affine;
        const auto layers = srs_layers(pv, 0xC0 ^ pv, &affine);
        const PreparedProverParam pp = be.prepare_prover_param(pv, layers);
        for (size_t nv = 0; nv <= pv; nv++) {
            const Table values = field_table(nv, 0xC1 ^ nv);
            const G1 expected = independent_commitment(affine, pv, nv, values);
            uint8_t cpu[96];
            CHECK(or_kzg_commit(affine[pv - nv].data(), values.data()->data(), nv, cpu) == 0);
            CHECK(packet_of(cpu) == expected);
            CHECK(be.commit(pp, be.mle_from_evaluations(nv, values)) == expected);
        }
    }
}

static void multi_commit_preserves_order_duplicates_and_empty_batch(const CudaBackend &be) {
    const size_t pv = 4;
    std::vector<std::vector<uint8_t>> affine;
    const PreparedProverParam pp = be.prepare_prover_param(pv, srs_layers(pv, 0x77, &affine));
    const Table constant = field_table(0, 0x01), two_a = field_table(2, 0x02), two_b = field_table(2, 0x04),
                four = field_table(4, 0x05);
    const Mle c = be.mle_from_evaluations(0, constant), a = be.mle_from_evaluations(2, two_a),
              dup = be.mle_from_evaluations(2, two_a), b = be.mle_from_evaluations(2, two_b),
              f = be.mle_from_evaluations(4, four);
    CHECK(a.id() != dup.id());
    CHECK(a.id() != b.id());
    const Mle a_clone = a;
    CHECK(a_clone.id() == a.id());
    const std::vector<G1> got = be.multi_commit(pp, {c, a, a_clone, dup, b, f});
    const std::vector<G1> expected = {independent_commitment(affine, pv, 0, constant),
                                      independent_commitment(affine, pv, 2, two_a),
                                      independent_commitment(affine, pv, 2, two_a),
                                      independent_commitment(affine, pv, 2, two_a),
                                      independent_commitment(affine, pv, 2, two_b),
                                      independent_commitment(affine, pv, 4, four)};
    CHECK(got == expected);
    CHECK(be.multi_commit(pp, {}).empty());
}

static void commit_and_open_reject_oversized_dimensions_and_mismatched_points(const CudaBackend &be) {
    const size_t pv = 2;
    std::vector<std::vector<uint8_t>> affine;
    const PreparedProverParam pp = be.prepare_prover_param(pv, srs_layers(pv, 0x88, &affine));
    for (size_t nv : {size_t(1), size_t(2), size_t(3)}) {
        const Table values = field_table(nv, 0x89);
        const Mle h = be.mle_from_evaluations(nv, values);
        std::vector<Fr> point;
        for (size_t i = 0; i < nv; i++) point.push_back(fr::from_u64(i + 2));
        if (nv > pv) {
            EXPECT_INVALID_PARAMETERS(be.commit(pp, h));
            EXPECT_INVALID_PARAMETERS(be.multi_commit(pp, {h}));
            EXPECT_INVALID_PARAMETERS(be.open(pp, h, point));
        } else {
            const std::vector<Fr> shorter(point.begin(), point.end() - 1);
            EXPECT_INVALID_PARAMETERS(be.open(pp, h, shorter));
            if (nv == pv) CHECK(be.open(pp, h, point).second == cpu_open(affine, pv, values, nv, point).second);
        }
    }
}

static void open_matches_cpu_with_exact_quotients_and_evaluations(const CudaBackend &be) {
    const size_t pv = 4;
    std::vector<std::vector<uint8_t>> affine;
    const PreparedProverParam pp = be.prepare_prover_param(pv, srs_layers(pv, 0x0C, &affine));
    for (size_t nv = 0; nv <= pv; nv++) {
        const Table values = field_table(nv, 0x0D ^ nv);
        const Mle h = be.mle_from_evaluations(nv, values);
        for (const auto &point : comparison_points(nv, 0x0E)) {
            const auto cpu = cpu_open(affine, pv, values, nv, point);
            const auto got = be.open(pp, h, point);
            CHECK(cpu.second == multilinear_eval(values, point));
            CHECK(got.second == cpu.second);
            CHECK(got.first == cpu.first);
            CHECK(got.first.size() == nv);
        }
    }
}

static void srs_ingress_rejects_invalid_layer_shapes(const CudaBackend &be) {
    const size_t pv = 2;
    const auto layers = srs_layers(pv, 0x5A, nullptr);
    EXPECT_INVALID_PARAMETERS(be.prepare_prover_param(pv, {layers.begin(), layers.begin() + pv}));
    auto extra = layers;
    extra.push_back(layers[0]);
    EXPECT_INVALID_PARAMETERS(be.prepare_prover_param(pv, extra));
    EXPECT_INVALID_PARAMETERS(be.prepare_prover_param(pv + 1, layers));
    auto shorter = layers;
    shorter[0].pop_back();
    EXPECT_INVALID_PARAMETERS(be.prepare_prover_param(pv, shorter));
    auto longer = layers;
    longer[pv].push_back(layers[0][0]);
    EXPECT_INVALID_PARAMETERS(be.prepare_prover_param(pv, longer));
    // an unknown tag, and a non-canonical coordinate (points themselves are
    // trusted, as in the reference: no curve or subgroup check on ingress)
    auto tag = layers;
    tag[0][1][0] = 2;
    EXPECT_INVALID_PARAMETERS(be.prepare_prover_param(pv, tag));
    auto big = layers;
    for (int i = 1; i <= 48; i++) big[0][2][i] = 0xff;
    EXPECT_INVALID_PARAMETERS(be.prepare_prover_param(pv, big));
}

static void identity_srs_base_is_accepted_and_commits_exactly(const CudaBackend &be) {
    const size_t pv = 2;
    std::vector<std::vector<uint8_t>> affine;
    auto layers = srs_layers(pv, 0x6B, &affine);
    layers[0][3] = G1{};
    layers[0][3][0] = 1;  // infinity packet
    std::memset(affine[0].data() + 96 * 3, 0, 96);
    const PreparedProverParam pp = be.prepare_prover_param(pv, layers);
    const Table values = field_table(pv, 0x6C);
    CHECK(be.commit(pp, be.mle_from_evaluations(pv, values)) == independent_commitment(affine, pv, pv, values));
    // only the identity base carries weight: the commitment is the identity
    Table only(4, fr::zero());
    only[3] = fr::from_u64(12345);
    G1 inf{};
    inf[0] = 1;
    CHECK(be.commit(pp, be.mle_from_evaluations(pv, only)) == inf);
}

// ---------------------------------------------------------------------------
// contexts and resource lifetimes
// ---------------------------------------------------------------------------

using Products = std::vector<std::pair<Fr, std::vector<size_t>>>;

static VirtualPolynomial build_virtual_polynomial(size_t nv, const Products &products, const std::vector<Mle> &h) {
    VirtualPolynomial vp(nv);
    for (const auto &p : products) {
        std::vector<Mle> list;
        for (size_t i : p.second) list.push_back(h[i]);
        vp.add_mle_list(list, p.first);
    }
    return vp;
}

// the host tables of the polynomial's flattened factors (by handle identity)
static std::vector<Table> flattened_tables(const VirtualPolynomial &vp, const std::vector<Mle> &handles,
                                           const std::vector<Table> &tables) {
    std::vector<Table> out;
    for (const Mle &f : vp.flattened_ml_extensions())
        for (size_t i = 0; i < handles.size(); i++)
            if (handles[i].id() == f.id()) {
                out.push_back(tables[i]);
                break;
            }
    return out;
}

static std::vector<std::vector<Fr>> sumcheck_transcript(const CudaBackend &be, SumCheckProverState &st, size_t nv,
                                                       const std::vector<Fr> &challenges) {
    std::vector<std::vector<Fr>> msgs{be.prove_round_and_update_state(st, std::nullopt)};
    for (size_t k = 1; k < nv; k++) msgs.push_back(be.prove_round_and_update_state(st, challenges[k - 1]));
    return msgs;
}

// the oracle (CPU backend) transcript of the same description
static std::vector<std::vector<Fr>> cpu_transcript(const VirtualPolynomial &vp, const std::vector<Table> &factors,
                                                   size_t nv, const std::vector<Fr> &challenges) {
    std::vector<size_t> offsets{0}, indices;
    std::vector<Fr> coefs;
    for (const auto &p : vp.products) {
        indices.insert(indices.end(), p.second.begin(), p.second.end());
        offsets.push_back(indices.size());
        coefs.push_back(p.first);
    }
    const auto fp = ptrs(factors);
    or_sumcheck *s = or_sumcheck_create(nv, vp.aux_info.max_degree, fp.data(), fp.size(),
                                        coefs.empty() ? nullptr : coefs.data()->data(), offsets.data(), coefs.size(),
                                        indices.empty() ? nullptr : indices.data(), indices.size());
    if (!s) fixture_failed("or_sumcheck_create");
    std::vector<std::vector<Fr>> msgs;
    for (size_t k = 0; k < nv; k++) {
        std::vector<Fr> m(vp.aux_info.max_degree + 1);
        if (or_sumcheck_round(s, k ? challenges[k - 1].data() : nullptr, m.data()->data()) != 0) {
            or_sumcheck_destroy(s);
            fixture_failed("or_sumcheck_round");
        }
        msgs.push_back(m);
    }
    or_sumcheck_destroy(s);
    return msgs;
}

// round messages from the definition: fold with the previous challenges, then
// s_k(t) = sum_b sum_p c_p prod_j (lo_j + t (hi_j - lo_j)) for t = 0..d
static std::vector<std::vector<Fr>> expected_messages(const Products &products, std::vector<Table> tables, size_t nv,
                                                      size_t degree, const std::vector<Fr> &challenges) {
    std::vector<std::vector<Fr>> msgs;
    for (size_t k = 0; k < nv; k++) {
        if (k > 0)
            for (Table &t : tables) {
                Table g(t.size() / 2);
                for (size_t b = 0; b < g.size(); b++)
                    g[b] = fr::add(t[2 * b], fr::mul(challenges[k - 1], fr::sub(t[2 * b + 1], t[2 * b])));
                t.swap(g);
            }
        const size_t half = size_t(1) << (nv - k - 1);
        std::vector<Fr> m(degree + 1, fr::zero());
        for (size_t t = 0; t <= degree; t++) {
            const Fr ft = fr::from_u64(t);
            for (size_t b = 0; b < half; b++)
                for (const auto &p : products) {
                    Fr v = p.first;
                    for (size_t j : p.second) {
                        const Table &f = tables[j];
                        v = fr::mul(v, fr::add(f[2 * b], fr::mul(ft, fr::sub(f[2 * b + 1], f[2 * b]))));
                    }
                    m[t] = fr::add(m[t], v);
                }
        }
        msgs.push_back(m);
    }
    return msgs;
}

static void independent_contexts_isolate_resources_without_masking_multicontext(const CudaBackend &first) {
    const CudaBackend second(0);
    const Table values = field_table(2, 0x2A);
    const Mle a = first.mle_from_evaluations(2, values), b = second.mle_from_evaluations(2, values);
    const std::vector<Fr> point = comparison_points(2, 0x2B)[0];
    const Fr expected = multilinear_eval(values, point);
    CHECK(first.evaluate(a, point) == expected);
    CHECK(second.evaluate(b, point) == expected);
    EXPECT_INVALID_PARAMETERS(first.evaluate(b, point));
    EXPECT_INVALID_PARAMETERS(second.evaluate(a, point));
    EXPECT_INVALID_PARAMETERS(first.linear_combination({a, b}, {fr::one(), fr::one()}));
    std::vector<std::vector<uint8_t>> affine;
    const auto layers = srs_layers(2, 0x2C, &affine);
    const PreparedProverParam p1 = first.prepare_prover_param(2, layers), p2 = second.prepare_prover_param(2, layers);
    const G1 want = independent_commitment(affine, 2, 2, values);
    CHECK(first.commit(p1, a) == want);
    CHECK(second.commit(p2, b) == want);
    EXPECT_INVALID_PARAMETERS(first.commit(p1, b));
    EXPECT_INVALID_PARAMETERS(first.commit(p2, a));
    EXPECT_INVALID_PARAMETERS(second.commit(p1, b));
    EXPECT_INVALID_PARAMETERS(first.open(p2, a, point));
    CHECK(first.evaluate(a, point) == expected);
    VirtualPolynomial vp(1);
    vp.add_mle_list({first.mle_from_evaluations(1, field_table(1, 0x2D))}, fr::one());
    SumCheckProverState st = first.prover_init(vp);
    EXPECT_INVALID_PARAMETERS(second.prove_round_and_update_state(st, std::nullopt));
    CHECK(first.prove_round_and_update_state(st, std::nullopt).size() == 2);
}

static void resources_survive_ordered_drops_and_same_device_reuse() {
    std::vector<Table> tables;
    for (uint64_t i = 0; i < 3; i++) tables.push_back(field_table(2, 0x3C + i));
    const Products products = {{fr::from_u64(2), {0, 1}}, {fr::from_u64(3), {2}}};
    const std::vector<Fr> challenges = {fr::from_u64(5), fr::from_u64(7)};
    std::optional<CudaBackend> be(std::in_place, 0);
    std::optional<PreparedProverParam> params(be->prepare_prover_param(2, srs_layers(2, 0x3A, nullptr)));
    std::optional<std::vector<Mle>> handles(upload_all(*be, 2, tables));
    std::optional<VirtualPolynomial> vp(build_virtual_polynomial(2, products, *handles));
    const auto cpu = cpu_transcript(*vp, flattened_tables(*vp, *handles, tables), 2, challenges);
    std::optional<SumCheckProverState> st(be->prover_init(*vp));
    params.reset();
    std::vector<std::vector<Fr>> msgs{be->prove_round_and_update_state(*st, std::nullopt)};
    vp.reset();
    handles.reset();  // the state keeps its inputs alive
    msgs.push_back(be->prove_round_and_update_state(*st, challenges[0]));
    CHECK(msgs == cpu);
    st.reset();
    const Table values = field_table(2, 0x3B);
    std::optional<Mle> alive(be->mle_from_evaluations(2, values));
    CHECK(be->download(*alive) == values);
    std::optional<Mle> extra(be->mle_from_evaluations(1, field_table(1, 0x3E)));
    be.reset();  // handles keep the context; it closes with the last of them
    alive.reset();
    extra.reset();
    const CudaBackend next(0);
    const Table nv2 = field_table(2, 0x3F);
    CHECK(next.download(next.mle_from_evaluations(2, nv2)) == nv2);
}

// ---------------------------------------------------------------------------
// sumcheck
// ---------------------------------------------------------------------------

static void sumcheck_input_handles_can_be_dropped_after_prover_init(const CudaBackend &be) {
    const size_t nv = 2;
    std::vector<Table> tables;
    for (uint64_t i = 0; i < 3; i++) tables.push_back(field_table(nv, 0x44 + i));
    const Products products = {{fr::from_u64(2), {0, 0}}, {fr::from_u64(5), {1, 2}}};
    const std::vector<Fr> challenges = {fr::from_u64(8), fr::from_u64(9)};
    std::optional<std::vector<Mle>> handles(upload_all(be, nv, tables));
    std::optional<VirtualPolynomial> vp(build_virtual_polynomial(nv, products, *handles));
    const auto cpu = cpu_transcript(*vp, flattened_tables(*vp, *handles, tables), nv, challenges);
    SumCheckProverState st = be.prover_init(*vp);
    vp.reset();
    handles.reset();
    CHECK(sumcheck_transcript(be, st, nv, challenges) == cpu);
}

static void sumcheck_round_messages_match_cpu_for_mixed_products(const CudaBackend &be) {
    const size_t nv = 3;
    const Table shared = field_table(nv, 0x61);
    const std::vector<Table> tables = {shared, field_table(nv, 0x62), field_table(nv, 0x63), field_table(nv, 0x64),
                                       field_table(nv, 0x65), shared};  // equal contents, distinct handles
    const Products products = {{fr::from_u64(2), {0, 0}},    {fr::from_u64(3), {0, 1}},  {fr::from_u64(5), {1, 5}},
                               {fr::from_u64(7), {2, 3, 4}}, {fr::from_u64(11), {5}}, {fr::zero(), {0, 2, 3}}};
    const auto handles = upload_all(be, nv, tables);
    CHECK(handles[0].id() != handles[5].id());
    const VirtualPolynomial vp = build_virtual_polynomial(nv, products, handles);
    CHECK(vp.aux_info.max_degree == 3);
    CHECK(vp.flattened_ml_extensions().size() == 6);
    const std::vector<std::vector<size_t>> want_idx = {{0, 0}, {0, 1}, {1, 2}, {3, 4, 5}, {2}, {0, 3, 4}};
    for (size_t p = 0; p < want_idx.size(); p++) CHECK(vp.products[p].second == want_idx[p]);
    const auto flat = flattened_tables(vp, handles, tables);
    Products flat_products;
    for (const auto &p : vp.products) flat_products.push_back(p);
    const std::vector<std::vector<Fr>> challenge_sets = {{fr_of(0x66, 0), fr_of(0x66, 1), fr_of(0x66, 2)},
                                                         {fr::zero(), fr::one(), fr::neg(fr::one())}};
    for (const auto &ch : challenge_sets) {
        const auto cpu = cpu_transcript(vp, flat, nv, ch);
        SumCheckProverState st = be.prover_init(vp);
        const auto got = sumcheck_transcript(be, st, nv, ch);
        CHECK(got == cpu);
        CHECK(got == expected_messages(flat_products, flat, nv, 3, ch));
    }
}

static void sumcheck_repeated_factors_mixed_arity_max_degree_34_are_independent(const CudaBackend &be) {
    const size_t nv = 3;
    std::vector<Table> tables;
    for (uint64_t i = 0; i < 7; i++) tables.push_back(field_table(nv, 0x71 + i));
    Products products;
    for (size_t arity = 1; arity <= 34; arity++) {
        std::vector<size_t> idx;
        for (size_t o = 0; o < arity; o++) idx.push_back((o * 3 + arity) % 7);
        products.push_back({fr::from_u64(arity + 1), idx});
    }
    products.push_back({fr::zero(), {0, 0, 0}});
    const auto handles = upload_all(be, nv, tables);
    const VirtualPolynomial vp = build_virtual_polynomial(nv, products, handles);
    CHECK(vp.aux_info.max_degree == 34);
    CHECK(vp.flattened_ml_extensions().size() == 7);
    const auto flat = flattened_tables(vp, handles, tables);
    const std::vector<Fr> ch = {fr::from_u64(2), fr::from_u64(3), fr::from_u64(5)};
    const auto cpu = cpu_transcript(vp, flat, nv, ch);
    SumCheckProverState s1 = be.prover_init(vp), s2 = be.prover_init(vp);
    const auto m1 = be.prove_round_and_update_state(s1, std::nullopt);
    CHECK(m1 == cpu[0]);
    const auto t2 = sumcheck_transcript(be, s2, nv, ch);
    CHECK(t2 == cpu);
    std::vector<std::vector<Fr>> t1{m1};
    for (size_t k = 1; k < nv; k++) t1.push_back(be.prove_round_and_update_state(s1, ch[k - 1]));
    CHECK(t1 == cpu);
    Products flat_products(vp.products.begin(), vp.products.end());
    CHECK(t2 == expected_messages(flat_products, flat, nv, 34, ch));
    for (size_t i = 0; i < tables.size(); i++) CHECK(be.download(handles[i]) == tables[i]);
}

static void sumcheck_rejects_zero_dimension_and_zero_degree(const CudaBackend &be) {
    VirtualPolynomial zero_dim(0);
    zero_dim.add_mle_list({be.mle_from_evaluations(0, field_table(0, 0x91))}, fr::one());
    EXPECT_INVALID_PARAMETERS(be.prover_init(zero_dim));
    const VirtualPolynomial zero_degree(2);
    EXPECT_INVALID_PARAMETERS(be.prover_init(zero_degree));
}

static void sumcheck_empty_whole_polynomial_messages_and_call_order_contract(const CudaBackend &be) {
    VirtualPolynomial empty(2);
    empty.aux_info.max_degree = 2;
    SumCheckProverState es = be.prover_init(empty);
    const auto et = sumcheck_transcript(be, es, 2, {fr::from_u64(3), fr::from_u64(4)});
    for (const auto &m : et) {
        CHECK(m.size() == 3);
        for (const Fr &v : m) CHECK(fr::is_zero(v));
    }
    const Table values = field_table(2, 0x81);
    const Mle h = be.mle_from_evaluations(2, values);
    VirtualPolynomial empty_product(2);
    empty_product.aux_info.max_degree = 2;
    empty_product.products.push_back({fr::one(), {}});
    EXPECT_INVALID_PARAMETERS(be.prover_init(empty_product));
    VirtualPolynomial arity(2);
    arity.add_mle_list({h}, fr::one());
    arity.products.push_back({fr::one(), {0, 0}});  // arity above max_degree 1
    EXPECT_INVALID_PARAMETERS(be.prover_init(arity));
    // 2f + 3f^2 over [2, 3, 5, 7] (the reference's known answer,
    // backend/src/cpu/sum_check.rs:239-246): [101, 194, 317] then, with r = 2,
    // [56, 261, 616]
    const Mle kat = be.mle_from_evaluations(2, {fr::from_u64(2), fr::from_u64(3), fr::from_u64(5), fr::from_u64(7)});
    VirtualPolynomial poly = VirtualPolynomial::new_from_mle(kat, fr::from_u64(2));
    poly.add_mle_list({kat, kat}, fr::from_u64(3));
    SumCheckProverState st = be.prover_init(poly);
    EXPECT_INVALID_STATE(be.prove_round_and_update_state(st, fr::from_u64(2)));  // first round takes no challenge
    CHECK(be.prove_round_and_update_state(st, std::nullopt) ==
          (std::vector<Fr>{fr::from_u64(101), fr::from_u64(194), fr::from_u64(317)}));
    EXPECT_INVALID_STATE(be.prove_round_and_update_state(st, std::nullopt));  // later rounds need one
    CHECK(be.prove_round_and_update_state(st, fr::from_u64(2)) ==
          (std::vector<Fr>{fr::from_u64(56), fr::from_u64(261), fr::from_u64(616)}));
    EXPECT_INVALID_STATE(be.prove_round_and_update_state(st, fr::from_u64(2)));  // exhausted
    CHECK(be.download(kat) == (Table{fr::from_u64(2), fr::from_u64(3), fr::from_u64(5), fr::from_u64(7)}));
}

// Not a port: the MSM autotuner (an extension of this backend) measures and
// re-prepares the layers without changing any commitment.
static void msm_autotune_keeps_commitments(const CudaBackend &be) {
    tuning::clear();
    const size_t pv = 8;
    std::vector<std::vector<uint8_t>> affine;
    const auto layers = srs_layers(pv, 0xA7, &affine);
    const PreparedProverParam pp = be.prepare_prover_param(pv, layers);
    const auto entries = be.msm_autotune(pp, {6, 8});
    CHECK(entries.size() == 2);
    for (const auto &e : entries) {
        const tuning::Geometry g = tuning::query(0, size_t(e.size));
        CHECK(e.mode == 0 && g.window_bits == e.window_bits && g.segment == e.segment && g.chunk == e.chunk);
        CHECK(e.tuned_ms > 0 && e.tuned_ms <= e.model_ms);
    }
    const auto shared = be.msm_autotune(pp, {3, 5, 6, 7}, 1);
    CHECK(shared.size() == 1 && shared[0].mode == 1 && tuning::query(1, size_t(shared[0].size)).chunk == shared[0].chunk);
    for (size_t nv = 0; nv <= pv; nv++) {
        const Table values = field_table(nv, 0xA8 ^ nv);
        CHECK(be.commit(pp, be.mle_from_evaluations(nv, values)) == independent_commitment(affine, pv, nv, values));
    }
    EXPECT_INVALID_PARAMETERS(be.msm_autotune(pp, {9}));  // more points than layer 0 holds
    tuning::clear();
}

// ---------------------------------------------------------------------------

int main() {
    std::setvbuf(stdout, nullptr, _IONBF, 0);
    or_set_threads(0);
    struct Case {
        const char *name;
        std::function<void(const CudaBackend &)> run;
    };
    const std::vector<Case> cases = {
        {"linear_combination_and_evaluate_match_cpu_for_all_dimensions",
         linear_combination_and_evaluate_match_cpu_for_all_dimensions},
        {"eq_polynomial_matches_closed_form_and_cpu", eq_polynomial_matches_closed_form_and_cpu},
        {"fraction_polynomial_matches_cpu_and_rejects_zero_denominators",
         fraction_polynomial_matches_cpu_and_rejects_zero_denominators},
        {"fraction_zero_detection_spans_grid_stride_tiles_without_poisoning",
         fraction_zero_detection_spans_grid_stride_tiles_without_poisoning},
        {"product_recurrence_and_factors_match_cpu", product_recurrence_and_factors_match_cpu},
        {"nums_and_denoms_match_cpu_with_nonidentity_permutations",
         nums_and_denoms_match_cpu_with_nonidentity_permutations},
        {"commit_matches_cpu_and_independent_msm", commit_matches_cpu_and_independent_msm},
        {"multi_commit_preserves_order_duplicates_and_empty_batch",
         multi_commit_preserves_order_duplicates_and_empty_batch},
        {"commit_and_open_reject_oversized_dimensions_and_mismatched_points",
         commit_and_open_reject_oversized_dimensions_and_mismatched_points},
        {"open_matches_cpu_with_exact_quotients_and_evaluations",
         open_matches_cpu_with_exact_quotients_and_evaluations},
        {"srs_ingress_rejects_invalid_layer_shapes", srs_ingress_rejects_invalid_layer_shapes},
        {"identity_srs_base_is_accepted_and_commits_exactly", identity_srs_base_is_accepted_and_commits_exactly},
        {"independent_contexts_isolate_resources_without_masking_multicontext",
         independent_contexts_isolate_resources_without_masking_multicontext},
        {"resources_survive_ordered_drops_and_same_device_reuse",
         [](const CudaBackend &) { resources_survive_ordered_drops_and_same_device_reuse(); }},
        {"sumcheck_input_handles_can_be_dropped_after_prover_init",
         sumcheck_input_handles_can_be_dropped_after_prover_init},
        {"sumcheck_round_messages_match_cpu_for_mixed_products", sumcheck_round_messages_match_cpu_for_mixed_products},
        {"sumcheck_repeated_factors_mixed_arity_max_degree_34_are_independent",
         sumcheck_repeated_factors_mixed_arity_max_degree_34_are_independent},
        {"sumcheck_rejects_zero_dimension_and_zero_degree", sumcheck_rejects_zero_dimension_and_zero_degree},
        {"msm_autotune_keeps_commitments", msm_autotune_keeps_commitments},
        {"sumcheck_empty_whole_polynomial_messages_and_call_order_contract",
         sumcheck_empty_whole_polynomial_messages_and_call_order_contract},
    };
    int failed_cases = 0;
    {
        const CudaBackend be(0);
        for (const Case &c : cases) {
            const int before = g_failures;
            try {
                c.run(be);
            } catch (const std::exception &e) {
                g_failures++;
                std::fprintf(stderr, "  unexpected exception: %s\n", e.what());
            }
            const bool ok = g_failures == before;
            failed_cases += ok ? 0 : 1;
            std::printf("%s %s\n", ok ? "ok    " : "FAILED", c.name);
        }
    }
    std::printf("%zu cases, %d failed; %d checks, %d failed\n", cases.size(), failed_cases, g_checks, g_failures);
    return g_failures == 0 ? 0 : 1;
}
