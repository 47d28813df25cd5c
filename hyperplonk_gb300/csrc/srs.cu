// srs.cu -- synthetic workload generation on the GPU machine: the testing SRS of
// subroutines/src/pcs/multilinear_kzg/srs.rs:158-235 (computed on the device)
// and uniform Fr fixtures (host).
//
// Fixture stream: ChaCha20 block function (RFC 8439) keyed by a 64-bit seed
// (key words 0-1 = seed, other key and nonce words 0); element i of a stream
// is Fr::from_le_bytes_mod_order of keystream block i (counter = low 32 bits
// of i, first nonce word = high 32 bits).  These streams do not reproduce
// arkworks' StdRng / Fr::rand.
//
// SRS: t_i = element i (i < nv), s = element nv, g = s * G1.  Layer i
// (i < nv) is g * eq(t[i..nv), x) over the 2^(nv-i) points x (t_i <-> bit 0);
// layer nv is [g].  The device evaluates every point with a 32 x 256 table of
// (d * 2^(8w) * s) * G1 (fixed-base comb: 32 mixed additions per point).
#include <algorithm>
#include <cstring>
#include <thread>
#include <vector>

#include "host_field.h"
#include "mle.cuh"
#include "msm.cuh"
#include "runtime.cuh"

using hp::check_cuda;
using hp::check_launch;
using hp::fail;
using hp::Fq;
using hp::Fr;
using hp::guard;
using hp::require;

namespace hp {

static inline uint32_t rotl32(uint32_t v, int n) { return (v << n) | (v >> (32 - n)); }

void chacha20_block(uint64_t seed, uint64_t index, uint8_t out[64]) {
    uint32_t s[16] = {0x61707865u, 0x3320646eu, 0x79622d32u, 0x6b206574u, uint32_t(seed), uint32_t(seed >> 32),
                      0, 0, 0, 0, 0, 0, uint32_t(index), uint32_t(index >> 32), 0, 0};
    uint32_t x[16];
    std::memcpy(x, s, sizeof x);
    auto qr = [&](int a, int b, int c, int d) {
        x[a] += x[b]; x[d] ^= x[a]; x[d] = rotl32(x[d], 16);
        x[c] += x[d]; x[b] ^= x[c]; x[b] = rotl32(x[b], 12);
        x[a] += x[b]; x[d] ^= x[a]; x[d] = rotl32(x[d], 8);
        x[c] += x[d]; x[b] ^= x[c]; x[b] = rotl32(x[b], 7);
    };
    for (int i = 0; i < 10; i++) {
        qr(0, 4, 8, 12); qr(1, 5, 9, 13); qr(2, 6, 10, 14); qr(3, 7, 11, 15);
        qr(0, 5, 10, 15); qr(1, 6, 11, 12); qr(2, 7, 8, 13); qr(3, 4, 9, 14);
    }
    for (int i = 0; i < 16; i++) {
        uint32_t v = x[i] + s[i];
        out[4 * i] = uint8_t(v);
        out[4 * i + 1] = uint8_t(v >> 8);
        out[4 * i + 2] = uint8_t(v >> 16);
        out[4 * i + 3] = uint8_t(v >> 24);
    }
}

static host::Fr64 fixture_element(uint64_t seed, uint64_t index) {
    uint8_t blk[64];
    chacha20_block(seed, index, blk);
    return host::from_wide64(blk);
}

__device__ __forceinline__ Affine generator_mont() {
    Fq x, y;
    constexpr uint32_t GX[12] = {0xdb22c6bbu, 0xfb3af00au, 0xf97a1aefu, 0x6c55e83fu, 0x171bac58u, 0xa14e3a3fu,
                                 0x9774b905u, 0xc3688c4fu, 0x4fa9ac0fu, 0x2695638cu, 0x3197d794u, 0x17f1d3a7u};
    constexpr uint32_t GY[12] = {0x46c5e7e1u, 0x0caa2329u, 0xa2888ae4u, 0xd03cc744u, 0x2c04b3edu, 0x00db18cbu,
                                 0xd5d00af6u, 0xfcf5e095u, 0x741d8ae4u, 0xa09e30edu, 0xe3aaa0f1u, 0x08b3f481u};
#pragma unroll
    for (int i = 0; i < 12; i++) {
        x.v[i] = GX[i];
        y.v[i] = GY[i];
    }
    Affine a;
    a.x = to_mont(x);
    a.y = to_mont(y);
    return a;
}

// table[w * 256 + d] = (d * 2^(8w) * s) * G1, XYZZ, by double-and-add.
__global__ void k_srs_table(Fr s, Xyzz *table) {
    int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= 32 * 256) return;
    int w = idx >> 8, d = idx & 255;
    Fr k = from_u32<FrParams>(uint32_t(d)) * s;
    Fr f256 = from_u32<FrParams>(256u);
    for (int i = 0; i < w; i++) k = k * f256;
    Fr kc = from_mont(k);
    Affine g = generator_mont();
    Xyzz acc = xyzz_inf();
    for (int bit = 255; bit >= 0; bit--) {
        acc = xyzz_double(acc);
        if ((kc.v[bit >> 5] >> (bit & 31)) & 1) acc = xyzz_add_affine(acc, g.x, g.y);
    }
    store_xyzz(&table[idx], acc);
}

// out[j] = e_j * g with e_j Montgomery scalars, via the comb table.
__global__ void k_srs_points(const Fr *scalars, size_t n, const Affine *table, Xyzz *out) {
    for (size_t j = blockIdx.x * size_t(blockDim.x) + threadIdx.x; j < n; j += size_t(gridDim.x) * blockDim.x) {
        Fr e = from_mont(load_fr(&scalars[j]));
        Xyzz acc = xyzz_inf();
        for (int w = 0; w < 32; w++) {
            uint32_t byte = (e.v[w >> 2] >> (8 * (w & 3))) & 0xff;
            if (byte == 0) continue;
            Affine a = load_affine(&table[w * 256 + byte]);
            acc = xyzz_add_affine(acc, a.x, a.y);
        }
        store_xyzz(&out[j], acc);
    }
}

__global__ void k_affine_to_packets(const Affine *pts, size_t n, uint8_t *out) {
    for (size_t j = blockIdx.x * size_t(blockDim.x) + threadIdx.x; j < n; j += size_t(gridDim.x) * blockDim.x) {
        Affine a = load_affine(&pts[j]);
        uint8_t *p = out + 97 * j;
        if (affine_is_inf(a)) {
            p[0] = 1;
            for (int k = 1; k < 97; k++) p[k] = 0;
            continue;
        }
        p[0] = 0;
        Fq x = from_mont(a.x), y = from_mont(a.y);
        for (int i = 0; i < 12; i++)
            for (int b = 0; b < 4; b++) {
                p[1 + 4 * i + b] = uint8_t(x.v[i] >> (8 * b));
                p[49 + 4 * i + b] = uint8_t(y.v[i] >> (8 * b));
            }
    }
}

}  // namespace hp

extern "C" HpCudaStatus hp_cuda_v1_fixture_random_fr(uint64_t seed, uint64_t first, size_t count,
                                                     uint8_t *out) {
    return guard([&] {
        require(count == 0 || out != nullptr);
        unsigned threads = std::max(1u, std::min(64u, std::thread::hardware_concurrency()));
        if (count < 4096) threads = 1;
        std::vector<std::thread> pool;
        size_t chunk = (count + threads - 1) / threads;
        for (unsigned t = 0; t < threads; t++) {
            size_t b = t * chunk, e = std::min(count, b + chunk);
            if (b >= e) break;
            pool.emplace_back([=] {
                for (size_t i = b; i < e; i++) hp::host::to_canonical(hp::fixture_element(seed, first + i), out + 32 * i);
            });
        }
        for (auto &th : pool) th.join();
    });
}

extern "C" HpCudaStatus hp_cuda_v1_srs_generate(HpCudaContext *ctx, size_t num_vars, uint64_t seed,
                                                uint8_t *out_packets, size_t point_count) {
    return guard([&] {
        hp::require_ctx(ctx);
        require(out_packets != nullptr && num_vars >= 1 && num_vars <= 26);
        const size_t total = (size_t(1) << (num_vars + 1)) - 1;
        require(point_count == total);
        std::vector<Fr> t(num_vars);
        for (size_t i = 0; i < num_vars; i++) {
            hp::host::Fr64 v = hp::fixture_element(seed, i);
            std::memcpy(t[i].v, v.v, 32);
        }
        hp::host::Fr64 sv = hp::fixture_element(seed, num_vars);
        Fr s;
        std::memcpy(s.v, sv.v, 32);
        // comb table
        hp::Scratch txyzz(ctx, 8192 * sizeof(hp::Xyzz)), table(ctx, 8192 * sizeof(hp::Affine));
        hp::Scratch pre(ctx, std::max<size_t>(total, 8192) * sizeof(Fq));
        hp::k_srs_table<<<64, 128, 0, ctx->stream>>>(s, txyzz.as<hp::Xyzz>());
        check_launch();
        hp::xyzz_to_affine(ctx, txyzz.as<hp::Xyzz>(), table.as<hp::Affine>(), pre.as<Fq>(), 8192);
        // scalars: eq(t[i..]) for every layer i < nv, then [1] for layer nv
        hp::Scratch tdev(ctx, num_vars * sizeof(Fr)), scal(ctx, total * sizeof(Fr));
        check_cuda(cudaMemcpyAsync(tdev.ptr, t.data(), num_vars * sizeof(Fr), cudaMemcpyHostToDevice, ctx->stream));
        size_t off = 0;
        for (size_t i = 0; i < num_vars; i++) {
            hp::build_eq(ctx, tdev.as<Fr>() + i, num_vars - i, scal.as<Fr>() + off);
            off += hp::table_len(num_vars - i);
        }
        hp::host::Fr64 one = hp::host::one();
        check_cuda(cudaMemcpyAsync(scal.as<Fr>() + off, one.v, sizeof(Fr), cudaMemcpyHostToDevice, ctx->stream));
        hp::Scratch pts(ctx, total * sizeof(hp::Xyzz)), aff(ctx, total * sizeof(hp::Affine));
        hp::k_srs_points<<<hp::grid_for(ctx, total, 128), 128, 0, ctx->stream>>>(scal.as<Fr>(), total,
                                                                                table.as<hp::Affine>(),
                                                                                pts.as<hp::Xyzz>());
        check_launch();
        hp::xyzz_to_affine(ctx, pts.as<hp::Xyzz>(), aff.as<hp::Affine>(), pre.as<Fq>(), total);
        hp::Scratch pk(ctx, total * 97);
        hp::k_affine_to_packets<<<hp::grid_for(ctx, total, 256), 256, 0, ctx->stream>>>(aff.as<hp::Affine>(),
                                                                                      total, pk.as<uint8_t>());
        check_launch();
        check_cuda(cudaMemcpyAsync(out_packets, pk.ptr, total * 97, cudaMemcpyDeviceToHost, ctx->stream));
        ctx->sync();
    });
}

// Vanilla-plonk fixture (full-prove workload): see include/hp_cuda.h.
// Selectors from stream `seed` elements [k n, (k+1) n) for q_L, q_R, q_M, q_C
// (k = 0..3); w1, w2 from stream `witness_seed` elements [4n, 5n) and [5n, 6n);
// w3 solves the gate.  selectors / permutation may be null (witnesses only).
// Wired variant (`wired`): w2[i] = w1[wire(i)] with wire(i) = (A i + B) mod n,
// A odd (a bijection of Z_n), B = seed * C + 1, and the permutation swaps w2
// cell i with w1 cell wire(i) (2-cycles; w3 cells fixed), so the copy
// constraints hold and are not the identity.
constexpr uint64_t kWireA = 0x9E3779B97F4A7C15ULL, kWireC = 0xD1B54A32D192ED03ULL;

static void vanilla_fixture(uint64_t seed, uint64_t witness_seed, size_t num_vars, uint8_t *selectors,
                            uint8_t *witnesses, uint8_t *permutation, bool wired = false) {
    {
        const size_t n = size_t(1) << num_vars;
        hp::host::Fr64 minus_one;
        {
            uint8_t b[32];
            hp::host::Fr64 one = hp::host::one();
            // -1 = r - 1 in canonical form
            const uint64_t rm1[4] = {0xffffffff00000000ULL, 0x53bda402fffe5bfeULL, 0x3339d80809a1d805ULL,
                                     0x73eda753299d7d48ULL};
            std::memcpy(b, rm1, 32);
            require(hp::host::from_canonical(b, minus_one));
            (void)one;
        }
        unsigned threads = std::max(1u, std::min(64u, std::thread::hardware_concurrency()));
        if (n < 4096) threads = 1;
        std::vector<std::thread> pool;
        size_t chunk = (n + threads - 1) / threads;
        for (unsigned t = 0; t < threads; t++) {
            size_t b = t * chunk, e = std::min(n, b + chunk);
            if (b >= e) break;
            pool.emplace_back([=] {
                using namespace hp::host;
                for (size_t i = b; i < e; i++) {
                    Fr64 ql = hp::fixture_element(seed, i), qr = hp::fixture_element(seed, n + i);
                    Fr64 qm = hp::fixture_element(seed, 2 * n + i), qc = hp::fixture_element(seed, 3 * n + i);
                    Fr64 w1 = hp::fixture_element(witness_seed, 4 * n + i);
                    const size_t wire = wired ? size_t((kWireA * i + seed * kWireC + 1) & (n - 1)) : i;
                    Fr64 w2 = wired ? hp::fixture_element(witness_seed, 4 * n + wire)
                                    : hp::fixture_element(witness_seed, 5 * n + i);
                    Fr64 w3 = add(add(mont_mul(ql, w1), mont_mul(qr, w2)), add(mont_mul(mont_mul(qm, w1), w2), qc));
                    const Fr64 sel[5] = {ql, qr, minus_one, qm, qc};
                    const Fr64 wit[3] = {w1, w2, w3};
                    if (selectors)
                        for (int k = 0; k < 5; k++) to_canonical(sel[k], selectors + (size_t(k) * n + i) * 32);
                    for (int k = 0; k < 3; k++) {
                        to_canonical(wit[k], witnesses + (size_t(k) * n + i) * 32);
                        if (!permutation) continue;
                        // sigma(cell): w1 cell wire -> w2 cell i, w2 cell i -> w1 cell wire
                        const size_t row = (wired && k == 0) ? wire : i;
                        const uint64_t label = !wired || k == 2 ? uint64_t(k) * n + i
                                               : k == 0       ? uint64_t(n) + i
                                                              : uint64_t(wire);
                        uint8_t *p = permutation + (size_t(k) * n + row) * 32;
                        std::memset(p, 0, 32);
                        std::memcpy(p, &label, 8);
                    }
                }
            });
        }
        for (auto &th : pool) th.join();
    }
}

extern "C" HpCudaStatus hp_cuda_v1_fixture_vanilla_plonk(uint64_t seed, size_t num_vars, uint8_t *selectors,
                                                         uint8_t *witnesses, uint8_t *permutation) {
    return guard([&] {
        require(selectors != nullptr && witnesses != nullptr && permutation != nullptr && num_vars <= 28);
        vanilla_fixture(seed, seed, num_vars, selectors, witnesses, permutation);
    });
}

extern "C" HpCudaStatus hp_cuda_v1_fixture_vanilla_plonk_wired(uint64_t seed, size_t num_vars, uint8_t *selectors,
                                                               uint8_t *witnesses, uint8_t *permutation) {
    return guard([&] {
        require(selectors != nullptr && witnesses != nullptr && permutation != nullptr && num_vars >= 1 &&
                num_vars <= 28);
        vanilla_fixture(seed, seed, num_vars, selectors, witnesses, permutation, true);
    });
}

extern "C" HpCudaStatus hp_cuda_v1_fixture_vanilla_plonk_witness(uint64_t circuit_seed, uint64_t witness_seed,
                                                                 size_t num_vars, uint8_t *witnesses) {
    return guard([&] {
        require(witnesses != nullptr && num_vars <= 28);
        vanilla_fixture(circuit_seed, witness_seed, num_vars, nullptr, witnesses, nullptr);
    });
}
