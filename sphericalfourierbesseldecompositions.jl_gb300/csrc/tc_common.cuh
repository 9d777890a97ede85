// tcgen05 building blocks shared by the tensor-core kernels: shared-memory
// matrix descriptors (no swizzle, K-major), the kind::f16 instruction
// descriptor, bounded mbarrier waits, bulk copies, MMA issue/commit, fences
// and TMEM loads.  Inline PTX for sm_103a.
#pragma once

#include <cstdint>

namespace sfb {
namespace tc {

constexpr uint32_t SPIN_LIMIT = 1u << 20;   // ~1 s of try_wait polling

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1 << 46;      // descriptor version for the sm_100 family; no swizzle, base offset 0
    return d;
}

// kind::f16 instruction descriptor: BF16 x BF16 -> F32, both operands K-major.
__device__ __forceinline__ uint32_t idesc_bf16(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

// Bounded wait for the given phase parity; false on timeout.  Each try
// suspends the thread until the phase completes or SFB_MBAR_HINT_NS passes,
// so waiting warps do not take issue slots from working ones.
#ifndef SFB_MBAR_HINT_NS
#define SFB_MBAR_HINT_NS 1000u
#endif
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity) {
    const uint32_t a = smem_u32(bar);
    for (uint32_t it = 0; it < SPIN_LIMIT; ++it) {
        uint32_t done;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n"
            " selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(a), "r"(parity), "r"((uint32_t)(SFB_MBAR_HINT_NS))
            : "memory");
        if (done) return true;
    }
    return false;
}

__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accum) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(
            tmem_d),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accum)
        : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t *bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void tmem_ld8(uint32_t taddr, float (&v)[8]) {
    uint32_t r[8];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
                 : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 8; ++i) v[i] = __uint_as_float(r[i]);
}

// ---- error-free slicing (block floating point, Ozaki et al.) -----------------
// A value with |x| < 2^E is written as four slices s_k, s_k = RN(r_k) on the
// grid 2^(E - 6 - 8k), r_0 = x, r_{k+1} = r_k - s_k, formed as (r + C_k) - C_k
// with C_k = 1.5 * 2^(E + 17 - 8k).  Every step is exact in FP32.  |s_0| <= 64
// grid units and, since |r_k| is at most half a unit of the grid before,
// |s_k| <= 128 units for k >= 1: at most 8 significant bits, which BF16 holds
// exactly (it holds the integers up to 256).

__device__ __forceinline__ float pow2f(int e) { return __int_as_float((127 + e) << 23); }   // -126 <= e <= 127

__device__ __forceinline__ void slice_consts(int E, float (&C)[4]) {
#pragma unroll
    for (int k = 0; k < 4; ++k) C[k] = 1.5f * pow2f(E + 17 - 8 * k);
}

// The same with an 8-bit leading slice: grid 2^(E - 7 - 8k), |s_k| <= 128
// units for every k.
__device__ __forceinline__ void slice_consts8(int E, float (&C)[4]) {
#pragma unroll
    for (int k = 0; k < 4; ++k) C[k] = 1.5f * pow2f(E + 16 - 8 * k);
}

__device__ __forceinline__ uint32_t bf16x2(float lo, float hi) {
    uint32_t r;
    asm("cvt.rn.bf16x2.f32 %0, %1, %2;" : "=r"(r) : "f"(hi), "f"(lo));
    return r;
}

// slices of the pair (x0, x1) packed as bf16x2 words w[k] (x0 in the low half)
__device__ __forceinline__ void slice_pair(float x0, float x1, const float (&C)[4], uint32_t (&w)[4]) {
    float r0 = x0, r1 = x1;
#pragma unroll
    for (int s = 0; s < 4; ++s) {
        const float a0 = __fsub_rn(__fadd_rn(r0, C[s]), C[s]);
        const float a1 = __fsub_rn(__fadd_rn(r1, C[s]), C[s]);
        w[s] = bf16x2(a0, a1);
        r0 = __fsub_rn(r0, a0);
        r1 = __fsub_rn(r1, a1);
    }
}

// Double-float source (x = hi + lo, |lo| <= ulp(hi)/2): the first slice comes
// from hi; the remainder (hi - s_0) + lo rounds at the last slice's unit.
__device__ __forceinline__ void slice_pair_df(float h0, float l0, float h1, float l1, const float (&C)[4],
                                              uint32_t (&w)[4]) {
    const float a0 = __fsub_rn(__fadd_rn(h0, C[0]), C[0]);
    const float a1 = __fsub_rn(__fadd_rn(h1, C[0]), C[0]);
    w[0] = bf16x2(a0, a1);
    float r0 = __fadd_rn(__fsub_rn(h0, a0), l0), r1 = __fadd_rn(__fsub_rn(h1, a1), l1);
#pragma unroll
    for (int s = 1; s < 4; ++s) {
        const float b0 = __fsub_rn(__fadd_rn(r0, C[s]), C[s]);
        const float b1 = __fsub_rn(__fadd_rn(r1, C[s]), C[s]);
        w[s] = bf16x2(b0, b1);
        r0 = __fsub_rn(r0, b0);
        r1 = __fsub_rn(r1, b1);
    }
}

// exponent E with |v| < 2^E for the largest magnitude v (0 for zero / non-finite)
__device__ __forceinline__ int scale_exp(float mx) {
    int E = 0;
    if (mx > 0.f && isfinite(mx)) E = ilogbf(mx) + 1;
    return E;
}

// The ten products (s_a, s_b), s_a + s_b <= 3, issued as six MMAs: products
// that share the A slice and land on adjacent levels go as one MMA of twice
// the N over two consecutive B planes (the planes are stored back to back, so
// the second plane's rows continue the first's at the same stride, and level v
// occupies TMEM columns [v LS, (v + 1) LS) for the kernel's level stride LS =
// N):  q0 A0 x [B0|B1] -> levels 0, 1;  q1 A0 x [B2|B3] -> 2, 3;
// q2 A1 x [B0|B1] -> 1, 2;  q3 A1 x B2 -> 3;  q4 A2 x [B0|B1] -> 2, 3;
// q5 A3 x B0 -> 3.  q0 and q1 write every level first (no accumulate on the
// first K step).  With 8-bit slice steps the dropped level-4 products are
// below 2^-32 of the leading ones.
constexpr int NMERGED = 6;
__device__ __forceinline__ int mg_a(int q) { return q < 2 ? 0 : q < 4 ? 1 : q < 5 ? 2 : 3; }
__device__ __forceinline__ int mg_b(int q) { return (q == 1 || q == 3) ? 2 : 0; }
__device__ __forceinline__ int mg_lvl(int q) { return q == 0 ? 0 : q == 2 ? 1 : (q == 1 || q == 4) ? 2 : 3; }
__device__ __forceinline__ bool mg_two(int q) { return q != 3 && q != 5; }
__device__ __forceinline__ bool mg_first(int q) { return q < 2; }

}  // namespace tc
}  // namespace sfb
