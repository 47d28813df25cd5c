// mle.cuh -- MLE kernel parameter types and host helpers shared across
// translation units (sumcheck and KZG reuse fold, eq and download).
#pragma once
#include <cstddef>
#include <cstdint>

#include "field.cuh"

struct HpCudaContext;

namespace hp {

// Inputs that ride in kernel parameters (no device-side pointer tables).
constexpr int kMaxList = 32;
struct FrPtrList {
    const Fr *p[kMaxList];
};
struct FrMutPtrList {
    Fr *p[kMaxList];
};
struct FrScalarList {
    Fr s[kMaxList];
};

// Canonical LE32 -> Montgomery Fr (InvalidParameters if not canonical).
Fr host_scalar(const uint8_t *canonical);
// Canonical scalars -> Montgomery, copied to a device array (synchronous).
void host_scalars_to_device(HpCudaContext *ctx, const uint8_t *canonical, size_t count, Fr *dst);
// In place canonical -> Montgomery on the context stream; non-canonical
// entries raise kFlagNonCanonical in the context status word.
void mle_to_mont_checked(HpCudaContext *ctx, Fr *data, size_t n);
// Device Montgomery table -> canonical host bytes (synchronous).
void download_canonical(HpCudaContext *ctx, const Fr *src, size_t n, uint8_t *out);
// Fix all nv variables (point[0] <-> bit 0) and leave the scalar at dst (device).
void fold_to_scalar(HpCudaContext *ctx, const Fr *table, size_t nv, const Fr *point, Fr *dst);
// eq(x, r) table for device-resident Montgomery r[0..nv).
void build_eq(HpCudaContext *ctx, const Fr *r_dev, size_t nv, Fr *out);
// prod(x) table from frac (reference compute_product_poly layout).
void product_tree(HpCudaContext *ctx, const Fr *frac, Fr *prod, size_t nv);

}  // namespace hp
