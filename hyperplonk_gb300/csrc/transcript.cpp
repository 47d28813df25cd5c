// transcript.cpp -- host Fiat-Shamir transcript: Merlin 1.0 framing over
// STROBE-128 over Keccak-f[1600].
//
// The reference's IOPTranscript (transcript/src/lib.rs:30-131) wraps the
// merlin 3.0.0 crate (pinned in Cargo.lock, not vendored).  This restates the
// published Merlin and STROBE-lite constructions: Transcript::new(label)
// = STROBE("Merlin v1.0") + append_message("dom-sep", label);
// append_message = meta-AD(label) + meta-AD(u32 LE length, more) + AD(msg);
// challenge_bytes = meta-AD(label) + meta-AD(u32 LE length, more) + PRF.
// Keccak-f[1600] follows FIPS 202; its round constants and rotation offsets
// are derived here from the spec's LFSR and (t+1)(t+2)/2 rules.
// Host only: the Fiat-Shamir transcript never touches the device, as at the
// reference's boundary (32-byte challenge in, round message out).
#include <cstdint>
#include <cstring>
#include <new>

#include "../../include/hp_cuda.h"
#include "transcript.h"

namespace {

struct KeccakTables {
    uint64_t rc[24];
    int rot[25];
    KeccakTables() {
        // round constants: rc(t) from the degree-8 LFSR x^8 + x^6 + x^5 + x^4 + 1
        auto rcbit = [](int t) {
            if (t % 255 == 0) return 1;
            uint32_t r = 1;
            for (int i = 1; i <= t % 255; i++) {
                r <<= 1;
                if (r & 0x100) r ^= 0x171;
            }
            return int(r & 1);
        };
        for (int ir = 0; ir < 24; ir++) {
            uint64_t c = 0;
            for (int j = 0; j <= 6; j++)
                if (rcbit(j + 7 * ir)) c |= uint64_t(1) << ((1 << j) - 1);
            rc[ir] = c;
        }
        // rotation offsets
        for (int i = 0; i < 25; i++) rot[i] = 0;
        int x = 1, y = 0;
        for (int t = 0; t < 24; t++) {
            rot[x + 5 * y] = ((t + 1) * (t + 2) / 2) % 64;
            int nx = y, ny = (2 * x + 3 * y) % 5;
            x = nx;
            y = ny;
        }
    }
};

const KeccakTables &tables() {
    static const KeccakTables t;
    return t;
}

inline uint64_t rotl(uint64_t v, int n) { return n == 0 ? v : (v << n) | (v >> (64 - n)); }

void keccak_f1600(uint64_t a[25]) {
    const KeccakTables &T = tables();
    for (int round = 0; round < 24; round++) {
        uint64_t c[5], d[5], b[25];
        for (int x = 0; x < 5; x++) c[x] = a[x] ^ a[x + 5] ^ a[x + 10] ^ a[x + 15] ^ a[x + 20];
        for (int x = 0; x < 5; x++) d[x] = c[(x + 4) % 5] ^ rotl(c[(x + 1) % 5], 1);
        for (int i = 0; i < 25; i++) a[i] ^= d[i % 5];
        // rho and pi: B[y, 2x+3y] = rot(A[x, y], r[x, y])
        for (int x = 0; x < 5; x++)
            for (int y = 0; y < 5; y++) b[y + 5 * ((2 * x + 3 * y) % 5)] = rotl(a[x + 5 * y], T.rot[x + 5 * y]);
        for (int y = 0; y < 5; y++)
            for (int x = 0; x < 5; x++)
                a[x + 5 * y] = b[x + 5 * y] ^ ((~b[(x + 1) % 5 + 5 * y]) & b[(x + 2) % 5 + 5 * y]);
        a[0] ^= T.rc[round];
    }
}

constexpr uint8_t kR = 166;  // STROBE-128 rate
constexpr uint8_t FLAG_I = 1, FLAG_A = 2, FLAG_C = 4, FLAG_T = 8, FLAG_M = 16, FLAG_K = 32;

struct Strobe128 {
    uint8_t st[200];
    uint8_t pos = 0, pos_begin = 0, cur_flags = 0;

    void permute() {
        uint64_t lanes[25];
        for (int i = 0; i < 25; i++) {
            uint64_t v = 0;
            for (int k = 7; k >= 0; k--) v = (v << 8) | st[8 * i + k];
            lanes[i] = v;
        }
        keccak_f1600(lanes);
        for (int i = 0; i < 25; i++)
            for (int k = 0; k < 8; k++) st[8 * i + k] = uint8_t(lanes[i] >> (8 * k));
    }
    void run_f() {
        st[pos] ^= pos_begin;
        st[pos + 1] ^= 0x04;
        st[kR + 1] ^= 0x80;
        permute();
        pos = 0;
        pos_begin = 0;
    }
    void absorb(const uint8_t *data, size_t n) {
        for (size_t i = 0; i < n; i++) {
            st[pos] ^= data[i];
            if (++pos == kR) run_f();
        }
    }
    void squeeze(uint8_t *out, size_t n) {
        for (size_t i = 0; i < n; i++) {
            out[i] = st[pos];
            st[pos] = 0;
            if (++pos == kR) run_f();
        }
    }
    bool begin_op(uint8_t flags, bool more) {
        if (more) return cur_flags == flags;
        if (flags & FLAG_T) return false;
        uint8_t old_begin = pos_begin;
        pos_begin = uint8_t(pos + 1);
        cur_flags = flags;
        uint8_t hdr[2] = {old_begin, flags};
        absorb(hdr, 2);
        bool force_f = (flags & (FLAG_C | FLAG_K)) != 0;
        if (force_f && pos != 0) run_f();
        return true;
    }
    void meta_ad(const uint8_t *d, size_t n, bool more) {
        begin_op(FLAG_M | FLAG_A, more);
        absorb(d, n);
    }
    void ad(const uint8_t *d, size_t n, bool more) {
        begin_op(FLAG_A, more);
        absorb(d, n);
    }
    void prf(uint8_t *out, size_t n, bool more) {
        begin_op(FLAG_I | FLAG_A | FLAG_C, more);
        squeeze(out, n);
    }
    explicit Strobe128(const uint8_t *label, size_t n) {
        std::memset(st, 0, sizeof st);
        const uint8_t init[6] = {1, uint8_t(kR + 2), 1, 0, 1, 96};
        std::memcpy(st, init, 6);
        std::memcpy(st + 6, "STROBEv1.0.2", 12);
        permute();
        meta_ad(label, n, false);
    }
};

}  // namespace

struct HpMerlinTranscript {
    Strobe128 strobe;
    explicit HpMerlinTranscript(const uint8_t *label, size_t n)
        : strobe(reinterpret_cast<const uint8_t *>("Merlin v1.0"), 11) {
        append(reinterpret_cast<const uint8_t *>("dom-sep"), 7, label, n);
    }
    void append(const uint8_t *label, size_t ln, const uint8_t *msg, size_t mn) {
        uint8_t len[4] = {uint8_t(mn), uint8_t(mn >> 8), uint8_t(mn >> 16), uint8_t(mn >> 24)};
        strobe.meta_ad(label, ln, false);
        strobe.meta_ad(len, 4, true);
        strobe.ad(msg, mn, false);
    }
    void challenge(const uint8_t *label, size_t ln, uint8_t *out, size_t on) {
        uint8_t len[4] = {uint8_t(on), uint8_t(on >> 8), uint8_t(on >> 16), uint8_t(on >> 24)};
        strobe.meta_ad(label, ln, false);
        strobe.meta_ad(len, 4, true);
        strobe.prf(out, on, false);
    }
};

namespace hp {
void merlin_append(HpMerlinTranscript *t, const char *label, const uint8_t *msg, size_t n) {
    t->append(reinterpret_cast<const uint8_t *>(label), std::strlen(label), msg, n);
}
void merlin_challenge(HpMerlinTranscript *t, const char *label, uint8_t *out, size_t n) {
    t->challenge(reinterpret_cast<const uint8_t *>(label), std::strlen(label), out, n);
}
}  // namespace hp

extern "C" HpCudaStatus hp_host_v1_merlin_new(const uint8_t *label, size_t label_len, HpMerlinTranscript **out) {
    if (!out || (label_len && !label) || label_len > 0xffffffffu) return HpCudaStatus{HP_CUDA_STATUS_INVALID_PARAMETERS, 0};
    *out = new (std::nothrow) HpMerlinTranscript(label, label_len);
    return *out ? HpCudaStatus{0, 0} : HpCudaStatus{HP_CUDA_STATUS_INVALID_STATE, 0};
}

extern "C" HpCudaStatus hp_host_v1_merlin_append(HpMerlinTranscript *t, const uint8_t *label, size_t label_len,
                                                 const uint8_t *msg, size_t msg_len) {
    if (!t || (label_len && !label) || (msg_len && !msg) || msg_len > 0xffffffffu)
        return HpCudaStatus{HP_CUDA_STATUS_INVALID_PARAMETERS, 0};
    t->append(label, label_len, msg, msg_len);
    return HpCudaStatus{0, 0};
}

extern "C" HpCudaStatus hp_host_v1_merlin_challenge(HpMerlinTranscript *t, const uint8_t *label, size_t label_len,
                                                    uint8_t *out, size_t out_len) {
    if (!t || (label_len && !label) || (out_len && !out) || out_len > 0xffffffffu)
        return HpCudaStatus{HP_CUDA_STATUS_INVALID_PARAMETERS, 0};
    t->challenge(label, label_len, out, out_len);
    return HpCudaStatus{0, 0};
}

extern "C" HpCudaStatus hp_host_v1_merlin_clone(const HpMerlinTranscript *t, HpMerlinTranscript **out) {
    if (!t || !out) return HpCudaStatus{HP_CUDA_STATUS_INVALID_PARAMETERS, 0};
    *out = new (std::nothrow) HpMerlinTranscript(*t);
    return *out ? HpCudaStatus{0, 0} : HpCudaStatus{HP_CUDA_STATUS_INVALID_STATE, 0};
}

extern "C" HpCudaStatus hp_host_v1_merlin_free(HpMerlinTranscript *t) {
    delete t;
    return HpCudaStatus{0, 0};
}

extern "C" HpCudaStatus hp_host_v1_keccak_f1600(uint8_t *state200) {
    if (!state200) return HpCudaStatus{HP_CUDA_STATUS_INVALID_PARAMETERS, 0};
    uint64_t lanes[25];
    for (int i = 0; i < 25; i++) {
        uint64_t v = 0;
        for (int k = 7; k >= 0; k--) v = (v << 8) | state200[8 * i + k];
        lanes[i] = v;
    }
    keccak_f1600(lanes);
    for (int i = 0; i < 25; i++)
        for (int k = 0; k < 8; k++) state200[8 * i + k] = uint8_t(lanes[i] >> (8 * k));
    return HpCudaStatus{0, 0};
}
