// The surrogate network on the fifth-generation tensor cores (tcgen05), 128 rows at a time.
//
// A warpgroup (128 threads) owns a tile of 128 queries, one row per thread. Every layer is one
// or more tcgen05.mma (kind::f16, BF16 operands, FP32 accumulation, M = 128) issued by the
// warpgroup's first thread, with the operands in shared memory and the accumulator in tensor
// memory (TMEM lane = row, column = output feature). Completion is signalled on an mbarrier by
// tcgen05.commit; the threads then read their row back with tcgen05.ld, apply SiLU in FP32, and
// write the BF16 activations as the next layer's A operand.
//
// The production form (mlp_tile_l1f) keeps layer 1 in FP32 on the CUDA cores, as training does,
// and runs layers 2, 3 and the output layer on the tensor cores. The all-tensor-core form
// (mlp_tile) moves the pieces that are FP32 on the CUDA cores into the MMAs as split BF16 products:
//   - layer 1: each input x = xh + xl and weight w = wh + wl (BF16 parts); the products
//     xh wh + xl wh + xh wl take 9 of the 16 K slots, the bias three more (below). The dropped
//     xl wl term is below 2^-18 of the product;
//   - biases: a constant A block whose rows are [1 1 1 0 ...] against a B block holding each
//     bias as hi + mid + lo BF16 parts (24 bits), one extra K step per layer;
//   - the output layer: W4 as three BF16 parts in the columns of an N = 16 tile, summed by the
//     thread after the read-back.
// Hidden weights and activations are BF16 as everywhere else; the weights are staged halved, so
// the accumulators are h = z / 2 and silu(z) = fma(h, tanh h, h).
//
// Shared-memory operands use the canonical K-major layout without swizzling: 8 x 16-byte core
// matrices of 128 contiguous bytes, K-adjacent core matrices 128 B apart (leading byte offset),
// 8-row groups kc * 128 B apart (stride byte offset), kc = 16-byte chunks per row. Each 16-byte
// chunk of a row is one st.shared.v4 by the thread that owns the row; the eight rows of a core
// matrix are eight consecutive threads, so the stores are bank-conflict free.
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "surrogate.cuh"

namespace bhr {
namespace surr {
namespace tc {

constexpr int kRows = 128;               // M of a tile: one row per thread of a warpgroup
constexpr uint32_t kTmemCols = 64;       // one N = 64 FP32 accumulator per warpgroup
constexpr long long kWaitCycles = 4000000000ll;  // about 2 s of SM clock before a wait gives up

// How a tile runs: the completion-wait limit in SM clocks, and (self-test only) whether the MMAs
// and their commit are withheld, so that every wait runs out with nothing in flight.
struct TileCtl {
    long long wait_cycles = kWaitCycles;
    bool withhold = false;
};

// byte offset of element (row, k) in a K-major no-swizzle tile with kc 16-byte chunks per row
__host__ __device__ constexpr uint32_t kmaj(int row, int k, int kc) {
    return uint32_t(((row >> 3) * kc + (k >> 3)) * 128 + (row & 7) * 16 + (k & 7) * 2);
}

struct Net {                  // shared memory, BF16 bit patterns in K-major tiles
    uint16_t w1[64 * 16];     // layer 1, n = feature: the split products and the bias (k = 9..11)
    uint16_t w2[64 * 64];     // [n = out][k = in], halved
    uint16_t w3[64 * 64];
    uint16_t b2[64 * 16];     // bias blocks: k = 0, 1, 2 hold hi, mid, lo
    uint16_t b3[64 * 16];
    uint16_t w4[16 * 64];     // n = 2 p + o: part p (hi, mid, lo) of output o's weights
    uint16_t b4[16 * 16];
    uint16_t ones[128 * 16];  // A block: every row [1 1 1 0 ... 0]
};
struct Tile {                 // per warpgroup
    uint16_t a[128 * 64];     // activations (8 chunks per row); the layer-1 block (2 chunks) aliases it
    unsigned long long mbar;
};

__device__ __forceinline__ uint16_t bf_bits(float v) { return __bfloat16_as_ushort(__float2bfloat16_rn(v)); }
__device__ __forceinline__ float bf_val(uint16_t b) { return __bfloat162float(__ushort_as_bfloat16(b)); }
__device__ __forceinline__ void split3(float v, uint16_t& h, uint16_t& m, uint16_t& l) {
    h = bf_bits(v);
    const float r1 = v - bf_val(h);
    m = bf_bits(r1);
    l = bf_bits(r1 - bf_val(m));
}
__device__ __forceinline__ uint32_t smem_u32(const void* p) { return uint32_t(__cvta_generic_to_shared(p)); }

// Stages the network (all threads of the block). fold: x1 is the same for every query and is
// folded into the layer-1 bias; the A rows' x1 slots then meet zero weights.
__device__ inline void load_net(Net& N, const float* __restrict__ P, bool fold, float x1) {
    const int nt = blockDim.x;
    for (int k = threadIdx.x; k < kH * kH; k += nt) {
        const int o = k / kH, i = k % kH;
        N.w2[kmaj(o, i, 8) / 2] = bf_bits(0.5f * P[kW2 + k]);
        N.w3[kmaj(o, i, 8) / 2] = bf_bits(0.5f * P[kW3 + k]);
    }
    for (int k = threadIdx.x; k < 64 * 16; k += nt) {
        const int n = k / 16, j = k % 16;
        N.w1[kmaj(n, j, 2) / 2] = 0;
        N.b2[kmaj(n, j, 2) / 2] = 0;
        N.b3[kmaj(n, j, 2) / 2] = 0;
    }
    for (int k = threadIdx.x; k < 16 * 64; k += nt) N.w4[kmaj(k / 64, k % 64, 8) / 2] = 0;
    for (int k = threadIdx.x; k < 16 * 16; k += nt) N.b4[kmaj(k / 16, k % 16, 2) / 2] = 0;
    for (int k = threadIdx.x; k < 128 * 16; k += nt) N.ones[kmaj(k / 16, k % 16, 2) / 2] = (k % 16) < 3 ? 0x3F80 : 0;
    __syncthreads();
    for (int f = threadIdx.x; f < kH; f += nt) {
        const float wa = fold ? 0.f : 0.5f * P[kW1 + 3 * f];
        const float wb = 0.5f * P[kW1 + 3 * f + 1], wc = 0.5f * P[kW1 + 3 * f + 2];
        const float b1 = 0.5f * (fold ? fmaf(P[kW1 + 3 * f], x1, P[kB1 + f]) : P[kB1 + f]);
        const float w[3] = {wa, wb, wc};
        for (int c = 0; c < 3; ++c) {  // slots 3c, 3c+1, 3c+2 meet xh, xl, xh
            const uint16_t h = bf_bits(w[c]), l = bf_bits(w[c] - bf_val(bf_bits(w[c])));
            N.w1[kmaj(f, 3 * c, 2) / 2] = h;
            N.w1[kmaj(f, 3 * c + 1, 2) / 2] = h;
            N.w1[kmaj(f, 3 * c + 2, 2) / 2] = l;
        }
        uint16_t h, m, l;
        split3(b1, h, m, l);
        N.w1[kmaj(f, 9, 2) / 2] = h;
        N.w1[kmaj(f, 10, 2) / 2] = m;
        N.w1[kmaj(f, 11, 2) / 2] = l;
        split3(0.5f * P[kB2 + f], h, m, l);
        N.b2[kmaj(f, 0, 2) / 2] = h;
        N.b2[kmaj(f, 1, 2) / 2] = m;
        N.b2[kmaj(f, 2, 2) / 2] = l;
        split3(0.5f * P[kB3 + f], h, m, l);
        N.b3[kmaj(f, 0, 2) / 2] = h;
        N.b3[kmaj(f, 1, 2) / 2] = m;
        N.b3[kmaj(f, 2, 2) / 2] = l;
        for (int o = 0; o < 2; ++o) {
            split3(P[kW4 + o * kH + f], h, m, l);
            N.w4[kmaj(o, f, 8) / 2] = h;
            N.w4[kmaj(2 + o, f, 8) / 2] = m;
            N.w4[kmaj(4 + o, f, 8) / 2] = l;
        }
    }
    if (threadIdx.x < 2) {
        uint16_t h, m, l;
        split3(P[kB4 + threadIdx.x], h, m, l);
        N.b4[kmaj(threadIdx.x, 0, 2) / 2] = h;
        N.b4[kmaj(threadIdx.x, 1, 2) / 2] = m;
        N.b4[kmaj(threadIdx.x, 2, 2) / 2] = l;
    }
}

// ---- tcgen05, TMEM and mbarrier primitives (PTX ISA, tcgen05 instructions)

// shared-memory matrix descriptor: start, leading and stride byte offsets (>> 4), the sm_100
// descriptor version (bit 46), no swizzling
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    return uint64_t((saddr >> 4) & 0x3FFFu) | (uint64_t((lbo >> 4) & 0x3FFFu) << 16) |
           (uint64_t((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}
// instruction descriptor for kind::f16: FP32 D (bits 4-5), BF16 A and B (7-9, 10-12), both
// K-major, N >> 3 at bits 17-22, M >> 4 at bits 24-28
__host__ __device__ constexpr uint32_t idesc_bf16(int m, int n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | (uint32_t(n >> 3) << 17) | (uint32_t(m >> 4) << 24);
}
__device__ __forceinline__ void mma(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
        :
        : "r"(tmem_d), "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
        : "memory");
}
// the mbarrier completes one phase once every MMA issued before by this thread has finished
__device__ __forceinline__ void commit(uint32_t mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar) : "memory");
}
__device__ __forceinline__ void mbar_init(uint32_t mbar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(mbar), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
// bounded wait for the phase with the given parity (non-blocking polls against a clock
// deadline); false if it did not complete
__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t parity, long long limit) {
    const long long t0 = clock64();
    for (;;) {
        uint32_t ok;
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(ok)
            : "r"(mbar), "r"(parity)
            : "memory");
        if (ok) return true;
        if (clock64() - t0 > limit) return false;
    }
}
__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// generic-proxy shared-memory writes made visible to the tensor cores' (async proxy) reads
__device__ __forceinline__ void fence_smem_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void wg_sync(int id) { asm volatile("bar.sync %0, 128;" ::"r"(id) : "memory"); }
// one warp: allocate / free TMEM columns (the base address is written to shared memory)
__device__ __forceinline__ void tmem_alloc(uint32_t slot, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(slot), "r"(ncols) : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
// this thread's TMEM lane, 32 consecutive columns from taddr; waits for the load in the same
// statement so that no use of the registers can be scheduled before it
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n\t"
        "tcgen05.wait::ld.sync.aligned;"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr)
        : "memory");
#pragma unroll
    for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}
__device__ __forceinline__ void tmem_ld8(uint32_t taddr, float (&v)[8]) {
    uint32_t r[8];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];\n\t"
        "tcgen05.wait::ld.sync.aligned;"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
        : "r"(taddr)
        : "memory");
#pragma unroll
    for (int i = 0; i < 8; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ uint32_t silu_pack(float lo, float hi) {
    float tl, th;
    asm("tanh.approx.f32 %0, %1;" : "=f"(tl) : "f"(lo));
    asm("tanh.approx.f32 %0, %1;" : "=f"(th) : "f"(hi));
    const __nv_bfloat162 v = __floats2bfloat162_rn(fmaf(lo, tl, lo), fmaf(hi, th, hi));
    return *reinterpret_cast<const uint32_t*>(&v);
}

// accumulator row (64 halved pre-activations) -> SiLU -> BF16 A row of the next layer
__device__ __forceinline__ void act_to_a(uint32_t taddr, unsigned char* a, int row) {
#pragma unroll
    for (int half = 0; half < 2; ++half) {
        float v[32];
        tmem_ld32(taddr + 32u * half, v);
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            uint4 w;
            w.x = silu_pack(v[8 * c + 0], v[8 * c + 1]);
            w.y = silu_pack(v[8 * c + 2], v[8 * c + 3]);
            w.z = silu_pack(v[8 * c + 4], v[8 * c + 5]);
            w.w = silu_pack(v[8 * c + 6], v[8 * c + 7]);
            *reinterpret_cast<uint4*>(a + kmaj(row, 32 * half + 8 * c, 8)) = w;
        }
    }
}

constexpr uint32_t kI64 = idesc_bf16(128, 64);
constexpr uint32_t kI16 = idesc_bf16(128, 16);

// Layer 1 in FP32 on the CUDA cores, as the training kernel computes it:
// per feature f, {w_x1, w_x2, w_sigma, b1} / 2 (halved, so that the pre-activation comes out as
// h = z / 2 and silu(z) = fma(h, tanh h, h)).
struct L1 {
    float4 w[kH];
};
__device__ inline void load_l1(L1& L, const float* __restrict__ P) {
    for (int f = threadIdx.x; f < kH; f += blockDim.x)
        L.w[f] = make_float4(0.5f * P[kW1 + 3 * f], 0.5f * P[kW1 + 3 * f + 1], 0.5f * P[kW1 + 3 * f + 2],
                             0.5f * P[kB1 + f]);
}

// The output layer and layers 2 and 3 on the tensor cores, from the A rows already in T.a;
// shared by both tile forms below. Returns false if a completion wait ran out.
__device__ inline bool mlp_tile_upper(const Net& N, Tile& T, uint32_t tmem, int row, int bar_id, uint32_t& phase,
                                      float2& out, const TileCtl& ctl) {
    unsigned char* a = reinterpret_cast<unsigned char*>(T.a);
    const uint32_t a_s = smem_u32(T.a), mbar = smem_u32(&T.mbar);
    const uint32_t taddr = tmem + (uint32_t((row >> 5) * 32) << 16);
    const bool issuer = row == 0 && !ctl.withhold;
    bool ok = true;
    const uint16_t* W[2] = {N.w2, N.w3};
    const uint16_t* B[2] = {N.b2, N.b3};
#pragma unroll 1
    for (int l = 0; l < 2; ++l) {  // layers 2 and 3
        fence_smem_async();
        fence_before();
        wg_sync(bar_id);
        if (issuer) {
            fence_after();
            const uint32_t w_s = smem_u32(W[l]);
#pragma unroll
            for (int s = 0; s < 4; ++s) mma(tmem, sdesc(a_s + 256u * s, 128, 1024), sdesc(w_s + 256u * s, 128, 1024), kI64, s);
            mma(tmem, sdesc(smem_u32(N.ones), 128, 256), sdesc(smem_u32(B[l]), 128, 256), kI64, 1u);
            commit(mbar);
        }
        ok &= mbar_wait(mbar, phase, ctl.wait_cycles);
        phase ^= 1u;
        fence_after();
        act_to_a(taddr, a, row);
    }
    // output layer: columns 2p + o hold part p of output o
    fence_smem_async();
    fence_before();
    wg_sync(bar_id);
    if (issuer) {
        fence_after();
        const uint32_t w_s = smem_u32(N.w4);
#pragma unroll
        for (int s = 0; s < 4; ++s) mma(tmem, sdesc(a_s + 256u * s, 128, 1024), sdesc(w_s + 256u * s, 128, 1024), kI16, s);
        mma(tmem, sdesc(smem_u32(N.ones), 128, 256), sdesc(smem_u32(N.b4), 128, 256), kI16, 1u);
        commit(mbar);
    }
    ok &= mbar_wait(mbar, phase, ctl.wait_cycles);
    phase ^= 1u;
    fence_after();
    float c[8];
    tmem_ld8(taddr, c);
    out = make_float2(c[0] + c[2] + c[4], c[1] + c[3] + c[5]);
    fence_before();
    return ok;
}

// One 128-row tile with layer 1 in FP32 on the CUDA cores (the same arithmetic, the same BF16
// activations as training) and layers 2, 3 and the output layer on the
// tensor cores. Called by all 128 threads of a warpgroup with their own row's query; the other
// arguments as mlp_tile's. The production form: the surrogate's tables and bhr_surrogate_eval.
__device__ inline bool mlp_tile_l1f(const Net& N, const L1& l1, Tile& T, uint32_t tmem, int row, int bar_id,
                                    uint32_t& phase, float4 x, float2& out, const TileCtl& ctl = TileCtl{}) {
    unsigned char* a = reinterpret_cast<unsigned char*>(T.a);
#pragma unroll
    for (int c = 0; c < 8; ++c) {  // features 8c .. 8c + 7: one 16-byte chunk of the row
        float h[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const float4 w = l1.w[8 * c + k];
            h[k] = fmaf(w.x, x.x, fmaf(w.y, x.y, fmaf(w.z, x.z, w.w)));
        }
        *reinterpret_cast<uint4*>(a + kmaj(row, 8 * c, 8)) =
            make_uint4(silu_pack(h[0], h[1]), silu_pack(h[2], h[3]), silu_pack(h[4], h[5]), silu_pack(h[6], h[7]));
    }
    return mlp_tile_upper(N, T, tmem, row, bar_id, phase, out, ctl);
}

// One 128-row tile through the network, called by all 128 threads of a warpgroup with their own
// row's query x = {x1, x2, sigma}; the warpgroup's named barrier is bar_id, its accumulator the
// TMEM columns from tmem (lane 0). phase tracks the tile mbarrier's parity. Returns false if an
// MMA did not complete within the bounded wait (every later step of the tile still runs, with
// bounded waits, so that the warpgroup's barriers stay matched).
__device__ inline bool mlp_tile(const Net& N, Tile& T, uint32_t tmem, int row, int bar_id, uint32_t& phase, float4 x,
                                float2& out, const TileCtl& ctl = TileCtl{}) {
    unsigned char* a = reinterpret_cast<unsigned char*>(T.a);
    const uint32_t a_s = smem_u32(T.a), mbar = smem_u32(&T.mbar);
    const uint32_t taddr = tmem + (uint32_t((row >> 5) * 32) << 16);
    const bool issuer = row == 0 && !ctl.withhold;
    bool ok = true;
    {  // layer-1 A row: x1h x1l x1h x2h x2l x2h sh sl sh 1 1 1 0 0 0 0
        const uint32_t x1h = bf_bits(x.x), x2h = bf_bits(x.y), sh = bf_bits(x.z);
        const uint32_t x1l = bf_bits(x.x - bf_val(uint16_t(x1h)));
        const uint32_t x2l = bf_bits(x.y - bf_val(uint16_t(x2h)));
        const uint32_t sl = bf_bits(x.z - bf_val(uint16_t(sh)));
        *reinterpret_cast<uint4*>(a + kmaj(row, 0, 2)) =
            make_uint4(x1h | (x1l << 16), x1h | (x2h << 16), x2l | (x2h << 16), sh | (sl << 16));
        *reinterpret_cast<uint4*>(a + kmaj(row, 8, 2)) = make_uint4(sh | (0x3F80u << 16), 0x3F803F80u, 0u, 0u);
    }
    fence_smem_async();
    fence_before();
    wg_sync(bar_id);
    if (issuer) {
        fence_after();
        mma(tmem, sdesc(a_s, 128, 256), sdesc(smem_u32(N.w1), 128, 256), kI64, 0u);
        commit(mbar);
    }
    ok &= mbar_wait(mbar, phase, ctl.wait_cycles);
    phase ^= 1u;
    fence_after();
    act_to_a(taddr, a, row);
    const uint16_t* W[2] = {N.w2, N.w3};
    const uint16_t* B[2] = {N.b2, N.b3};
#pragma unroll 1
    for (int l = 0; l < 2; ++l) {  // layers 2 and 3
        fence_smem_async();
        fence_before();
        wg_sync(bar_id);
        if (issuer) {
            fence_after();
            const uint32_t w_s = smem_u32(W[l]);
#pragma unroll
            for (int s = 0; s < 4; ++s) mma(tmem, sdesc(a_s + 256u * s, 128, 1024), sdesc(w_s + 256u * s, 128, 1024), kI64, s);
            mma(tmem, sdesc(smem_u32(N.ones), 128, 256), sdesc(smem_u32(B[l]), 128, 256), kI64, 1u);
            commit(mbar);
        }
        ok &= mbar_wait(mbar, phase, ctl.wait_cycles);
        phase ^= 1u;
        fence_after();
        act_to_a(taddr, a, row);
    }
    // output layer: columns 2p + o hold part p of output o
    fence_smem_async();
    fence_before();
    wg_sync(bar_id);
    if (issuer) {
        fence_after();
        const uint32_t w_s = smem_u32(N.w4);
#pragma unroll
        for (int s = 0; s < 4; ++s) mma(tmem, sdesc(a_s + 256u * s, 128, 1024), sdesc(w_s + 256u * s, 128, 1024), kI16, s);
        mma(tmem, sdesc(smem_u32(N.ones), 128, 256), sdesc(smem_u32(N.b4), 128, 256), kI16, 1u);
        commit(mbar);
    }
    ok &= mbar_wait(mbar, phase, ctl.wait_cycles);
    phase ^= 1u;
    fence_after();
    float c[8];
    tmem_ld8(taddr, c);
    out = make_float2(c[0] + c[2] + c[4], c[1] + c[3] + c[5]);
    fence_before();
    return ok;
}

}  // namespace tc
}  // namespace surr
}  // namespace bhr
