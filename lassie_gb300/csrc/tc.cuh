// Tensor-core (tcgen05) helpers for the rank-32 updates of the Gauss-Jordan
// factorisation: D[128 x NT] = A[128 x 32] * B[32 x NT] in FP32, in one of
// two forms:
//   * TF32 MMAs with the operands split as x = hi + lo (hi = x rounded to
//     TF32, lo = x - hi, exact), D = Ah*Bh + Ah*Bl + Al*Bh: three MMAs per
//     8-wide K step, close to an FP32 product (the dropped Al*Bl term is
//     below 2^-22 relative);
//   * BF16 operands (x rounded to nearest BF16), FP32 accumulation: one
//     kind::f16 MMA per 16-wide K step, each product exact and rounded once
//     into the FP32 sum -- the operands carry 8 significant bits, so the
//     factors are good to about 2^-9 and the FP64 refinement does the rest.
// Included by compat_engine.cu inside its namespace.
//
// Operands sit in shared memory in the canonical K-major layout without
// swizzling: 8-row x 16-byte core matrices, core matrices adjacent in K
// 128 bytes apart (leading byte offset), 8-row groups (K / 4) * 128 bytes
// apart (stride byte offset).  One elected thread issues the MMAs and commits
// them to an mbarrier; the accumulator lives in tensor memory and the four
// warps of a warpgroup read it back with tcgen05.ld (warp w % 4 reads lanes
// 32 * (w % 4) ...).  Every wait is bounded: a wait that runs out sets the
// caller's error flag and returns.
#pragma once

constexpr int kTcM = 128;   // rows of one MMA tile (TMEM lanes)
constexpr int kTcK = 32;    // panel width: four K = 8 TF32 MMAs
constexpr int kTcN = 128;   // columns of one MMA tile

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// x rounded to TF32 (10 explicit mantissa bits, ties away from zero in the
// dropped 13 bits); finite inputs only need this, inf/NaN pass unchanged.
__device__ __forceinline__ float tf32_hi(float x) {
    uint32_t b = __float_as_uint(x);
    if ((b & 0x7f800000u) == 0x7f800000u) return x;
    b = (b + 0x1000u) & 0xffffe000u;
    return __uint_as_float(b);
}

// Shared-memory matrix descriptor, K-major, no swizzle.
__device__ __forceinline__ uint64_t tc_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3fffu);
    d |= (uint64_t)((lbo >> 4) & 0x3fffu) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3fffu) << 32;
    d |= (uint64_t)1 << 46;  // descriptor version
    return d;                // base offset 0, relative leading offset, no swizzle
}

// Instruction descriptor: kind::tf32, D in FP32, A and B TF32 and K-major,
// M = kTcM, N = n.
__device__ __forceinline__ uint32_t tc_idesc_tf32(int n) {
    uint32_t d = 0;
    d |= 1u << 4;                    // D format: F32
    d |= 2u << 7;                    // A format: TF32
    d |= 2u << 10;                   // B format: TF32
    d |= (uint32_t)(n >> 3) << 17;   // N / 8
    d |= (uint32_t)(kTcM >> 4) << 24;  // M / 16
    return d;
}

// Byte offset of element (r, k) of a rows x 32 K-major operand.
__device__ __forceinline__ int tc_off(int r, int k) {
    return (r >> 3) * (kTcK / 4) * 128 + (k >> 2) * 128 + (r & 7) * 16 + (k & 3) * 4;
}

// The same for 16-bit elements: a core matrix row holds 8 elements of K.
__device__ __forceinline__ int tc_off16(int r, int k) {
    return (r >> 3) * (kTcK / 8) * 128 + (k >> 3) * 128 + (r & 7) * 16 + (k & 7) * 2;
}

// Instruction descriptor: kind::f16, D in FP32, A and B BF16 and K-major,
// M = kTcM, N = n.
__device__ __forceinline__ uint32_t tc_idesc_bf16(int n) {
    uint32_t d = 0;
    d |= 1u << 4;                      // D format: F32
    d |= 1u << 7;                      // A format: BF16
    d |= 1u << 10;                     // B format: BF16
    d |= (uint32_t)(n >> 3) << 17;     // N / 8
    d |= (uint32_t)(kTcM >> 4) << 24;  // M / 16
    return d;
}

// x rounded to the nearest BF16 (ties to even), as its 16 bits; inf/NaN
// keep their class.
__device__ __forceinline__ uint16_t bf16_bits(float x) {
    uint32_t b = __float_as_uint(x);
    if ((b & 0x7f800000u) == 0x7f800000u)
        return (uint16_t)((b >> 16) | ((b & 0xffffu) ? 0x40u : 0u));
    b += 0x7fffu + ((b >> 16) & 1u);
    return (uint16_t)(b >> 16);
}

__device__ __forceinline__ void tc_mbar_init(uint64_t *bar) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(bar)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// Bounded wait for the mbarrier phase `parity`; false if it ran out.
__device__ __forceinline__ bool tc_mbar_wait(uint64_t *bar, uint32_t parity) {
    const uint32_t a = smem_u32(bar);
    for (int it = 0; it < (1 << 22); it++) {
        uint32_t done;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
            " selp.u32 %0, 1, 0, p;\n}"
            : "=r"(done)
            : "r"(a), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

// One warp: allocate `ncols` TMEM columns, address to *slot (shared).
__device__ __forceinline__ void tc_alloc(uint32_t *slot, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(slot)),
                 "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tc_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols)
                 : "memory");
}

__device__ __forceinline__ void tc_mma_tf32(uint32_t dtmem, uint64_t adesc, uint64_t bdesc,
                                            uint32_t idesc, uint32_t accumulate) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}" ::"r"(dtmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}

__device__ __forceinline__ void tc_mma_f16(uint32_t dtmem, uint64_t adesc, uint64_t bdesc,
                                           uint32_t idesc, uint32_t accumulate) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(dtmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}

__device__ __forceinline__ void tc_commit(uint64_t *bar) {
    asm volatile(
        "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
            smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ void tc_fence_before() {
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_proxy_fence() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// 32 consecutive FP32 columns of this thread's TMEM lane.
__device__ __forceinline__ void tc_ld32(uint32_t taddr, float *v) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,"
        "%14,%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
          "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
          "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]),
          "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]),
          "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr)
        : "memory");
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 32; i++) v[i] = __uint_as_float(r[i]);
}

// Shared-memory footprint of one split tile: A hi/lo (128 x 32) and B hi/lo
// (kTcN x 32), FP32 each, plus the mbarrier and the TMEM address slot.
constexpr int kTcSmemBytes = 2 * kTcM * kTcK * 4 + 2 * kTcN * kTcK * 4 + 64;

// D = A * B for one tile by the whole CTA (kThreads = 512 threads).  The
// caller has stored the split operands with tc_off (sAh/sAl: A as 128 x 32,
// sBh/sBl: B as kTcN x 32, both K-major) and made them visible to the tensor
// core (tc_proxy_fence by the writers, then __syncthreads).  Thread t reads
// back row 32 * ((t / 32) % 4) + t % 32, columns 32 * (t / 128) + [0, 32) of
// D into out[32] (a warp may only read its quarter of the TMEM lanes, the
// four warpgroups take the four 32-column chunks).  tmem: kTcN allocated
// columns; phase: the mbarrier parity, flipped here.  Returns (uniformly)
// false if the MMA completion wait ran out.
__device__ __forceinline__ bool tc_tile_product(const float *sAh, const float *sAl,
                                                const float *sBh, const float *sBl,
                                                uint64_t *bar, uint32_t tmem, uint32_t &phase,
                                                float *out) {
    static_assert(kThreads == 4 * kTcN, "four warpgroups, one 32-column chunk each");
    const int tid = threadIdx.x;
    if (tid == 0) {
        tc_fence_after();
        const uint32_t idesc = tc_idesc_tf32(kTcN);
        const uint32_t sbo = (kTcK / 4) * 128;
        uint32_t acc = 0;
#pragma unroll
        for (int ks = 0; ks < kTcK / 8; ks++) {
            const uint32_t koff = ks * 2 * 128;  // two core matrices per K = 8 step
            const uint64_t ah = tc_desc(smem_u32(sAh) + koff, 128, sbo);
            const uint64_t al = tc_desc(smem_u32(sAl) + koff, 128, sbo);
            const uint64_t bh = tc_desc(smem_u32(sBh) + koff, 128, sbo);
            const uint64_t bl = tc_desc(smem_u32(sBl) + koff, 128, sbo);
            tc_mma_tf32(tmem, ah, bh, idesc, acc);
            acc = 1;
            tc_mma_tf32(tmem, ah, bl, idesc, 1);
            tc_mma_tf32(tmem, al, bh, idesc, 1);
        }
        tc_commit(bar);
    }
    const bool ok = tc_mbar_wait(bar, phase);
    tc_fence_after();
    if (ok) {
        const int w = tid >> 5, quad = w & 3, chunk = w >> 2;
        tc_ld32(tmem + ((uint32_t)(quad * 32) << 16) + chunk * 32, out);
    }
    phase ^= 1u;
    tc_fence_before();
    return __syncthreads_and(ok) != 0;
}

// Deeper products D = sum over K chunks of A_c * B_c (K = 32 per chunk), the
// accumulator staying in tensor memory.  The caller stages each chunk's
// operands as for tc_tile_product and makes them visible to the tensor core;
// thread 0 issues the chunk's MMAs and commits them (tc_chunk_issue*, first
// chunk: accumulate = false); every thread later waits for that commit
// (tc_chunk_wait: bounded, flips phase, uniformly false if the wait ran out),
// after which the chunk's shared-memory operands may be overwritten -- so a
// caller with two operand buffers stages the next chunk while the tensor
// core works on this one.  tc_tile_read reads the product back (same
// thread-to-entry map as tc_tile_product).
__device__ __forceinline__ void tc_chunk_issue(const float *sAh, const float *sAl,
                                               const float *sBh, const float *sBl, uint64_t *bar,
                                               uint32_t tmem, bool accumulate) {
    if (threadIdx.x == 0) {
        tc_fence_after();
        const uint32_t idesc = tc_idesc_tf32(kTcN);
        const uint32_t sbo = (kTcK / 4) * 128;
        uint32_t acc = accumulate ? 1u : 0u;
#pragma unroll
        for (int ks = 0; ks < kTcK / 8; ks++) {
            const uint32_t koff = ks * 2 * 128;
            const uint64_t ah = tc_desc(smem_u32(sAh) + koff, 128, sbo);
            const uint64_t al = tc_desc(smem_u32(sAl) + koff, 128, sbo);
            const uint64_t bh = tc_desc(smem_u32(sBh) + koff, 128, sbo);
            const uint64_t bl = tc_desc(smem_u32(sBl) + koff, 128, sbo);
            tc_mma_tf32(tmem, ah, bh, idesc, acc);
            acc = 1;
            tc_mma_tf32(tmem, ah, bl, idesc, 1);
            tc_mma_tf32(tmem, al, bh, idesc, 1);
        }
        tc_commit(bar);
    }
}

__device__ __forceinline__ void tc_chunk_issue_bf16(const uint16_t *sA, const uint16_t *sB,
                                                    uint64_t *bar, uint32_t tmem, bool accumulate) {
    if (threadIdx.x == 0) {
        tc_fence_after();
        const uint32_t idesc = tc_idesc_bf16(kTcN);
        const uint32_t sbo = (kTcK / 8) * 128;
#pragma unroll
        for (int ks = 0; ks < kTcK / 16; ks++) {
            const uint32_t koff = ks * 2 * 128;
            const uint64_t a = tc_desc(smem_u32(sA) + koff, 128, sbo);
            const uint64_t b = tc_desc(smem_u32(sB) + koff, 128, sbo);
            tc_mma_f16(tmem, a, b, idesc, (accumulate || ks > 0) ? 1u : 0u);
        }
        tc_commit(bar);
    }
}

__device__ __forceinline__ bool tc_chunk_wait(uint64_t *bar, uint32_t &phase) {
    const bool ok = tc_mbar_wait(bar, phase);
    tc_fence_after();
    phase ^= 1u;
    return __syncthreads_and(ok) != 0;
}

__device__ __forceinline__ void tc_tile_read(uint32_t tmem, float *out) {
    const int w = threadIdx.x >> 5, quad = w & 3, chunk = w >> 2;
    tc_ld32(tmem + ((uint32_t)(quad * 32) << 16) + chunk * 32, out);
    tc_fence_before();
    __syncthreads();
}

// The BF16 form: sA (A as 128 x 32) and sB (B as kTcN x 32) hold BF16 bits
// stored with tc_off16; otherwise as tc_tile_product (two MMAs, K = 16 each).
__device__ __forceinline__ bool tc_tile_product_bf16(const uint16_t *sA, const uint16_t *sB,
                                                     uint64_t *bar, uint32_t tmem,
                                                     uint32_t &phase, float *out) {
    static_assert(kThreads == 4 * kTcN, "four warpgroups, one 32-column chunk each");
    const int tid = threadIdx.x;
    if (tid == 0) {
        tc_fence_after();
        const uint32_t idesc = tc_idesc_bf16(kTcN);
        const uint32_t sbo = (kTcK / 8) * 128;
#pragma unroll
        for (int ks = 0; ks < kTcK / 16; ks++) {
            const uint32_t koff = ks * 2 * 128;  // two core matrices per K = 16 step
            const uint64_t a = tc_desc(smem_u32(sA) + koff, 128, sbo);
            const uint64_t b = tc_desc(smem_u32(sB) + koff, 128, sbo);
            tc_mma_f16(tmem, a, b, idesc, ks > 0 ? 1u : 0u);
        }
        tc_commit(bar);
    }
    const bool ok = tc_mbar_wait(bar, phase);
    tc_fence_after();
    if (ok) {
        const int w = tid >> 5, quad = w & 3, chunk = w >> 2;
        tc_ld32(tmem + ((uint32_t)(quad * 32) << 16) + chunk * 32, out);
    }
    phase ^= 1u;
    tc_fence_before();
    return __syncthreads_and(ok) != 0;
}
