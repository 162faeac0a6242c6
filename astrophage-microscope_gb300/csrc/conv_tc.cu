// conv_tc.cu -- 3x3x3 "same" convolutions on the 5th-generation tensor cores
// (tcgen05), for the learned field surrogate.
//
// Layout: activations are channels-last BF16, [D][H][W][C]; weights are
// [27 taps][Cout][Cin] BF16 with tap t = (dz+1)*9 + (dy+1)*3 + (dx+1).
//
// Forward (and input gradient, which for a stride-1 convolution is the same
// convolution with the weights flipped and transposed): implicit GEMM with
// M = 128 output voxels per CTA, N = Cout, K = 27 taps x Cin. For every tap
// a TMA copy brings the 128 voxels' input rows, shifted by the tap, straight
// from the channels-last tensor (the copy's zero fill outside the grid is the
// convolution's zero padding), and a second copy brings that tap's weights.
// One elected thread issues tcgen05.mma into an FP32 accumulator in tensor
// memory; four warps read it back (tcgen05.ld) and apply bias, ReLU, an
// optional gradient mask, and the output conversion.
//
// Weight gradient: dW[t] = dY^T X_t reduces over voxels, so K = voxels. Both
// operands are staged K-major from channel-major copies: dY^T [Cout][voxels]
// and three copies of X^T shifted by dx = -1, 0, +1 along x (a TMA copy's
// innermost coordinate must stay 16-byte aligned, so the one-voxel x shift is
// done once in memory; the y and z shifts are coordinates of the copy).
// CTAs split the voxels; partial sums are reduced in a fixed order, so the
// gradient is deterministic.
//
// Every wait is bounded. A role whose wait runs out raises the CTA's abort
// flag and the error word; the others see the flag and stop; the CTA then
// waits (bounded) for its own copies and MMAs in flight and frees its tensor
// memory before it exits.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "nn.h"

namespace agb {
namespace nn {
namespace {

constexpr int BM = 128;                 // output rows (voxels or channels) per CTA
constexpr int NST = 4;                  // pipeline stages
constexpr uint32_t SPIN_LIMIT = 1u << 24;

__device__ __forceinline__ uint32_t saddr(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void bar_init(uint64_t* b, uint32_t n) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(saddr(b)), "r"(n));
}
__device__ __forceinline__ void bar_expect(uint64_t* b, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(saddr(b)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool bar_try(uint64_t* b, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(saddr(b)), "r"(parity)
        : "memory");
    return ok != 0;
}
// Bounded wait that also gives up when another role raised the abort flag.
__device__ bool bar_wait(uint64_t* b, uint32_t parity, volatile int* abort_flag, uint32_t* err, uint32_t code) {
    for (uint32_t i = 0; i < SPIN_LIMIT; ++i) {
        if (bar_try(b, parity)) return true;
        if ((i & 255u) == 255u && *abort_flag) return false;
    }
    *abort_flag = 1;
    atomicCAS(err, 0u, code);
    return false;
}
// Bounded wait used on the way out (no abort check: it drains).
__device__ void bar_drain(uint64_t* b, uint32_t parity) {
    for (uint32_t i = 0; i < SPIN_LIMIT; ++i)
        if (bar_try(b, parity)) return;
}

__device__ __forceinline__ void tma3(void* dst, const CUtensorMap* m, uint64_t* b, int c0, int c1, int c2) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];"
        ::"r"(saddr(dst)), "l"(reinterpret_cast<uint64_t>(m)), "r"(c0), "r"(c1), "r"(c2), "r"(saddr(b))
        : "memory");
}
__device__ __forceinline__ void tma4(void* dst, const CUtensorMap* m, uint64_t* b, int c0, int c1, int c2, int c3) {
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], [%6];"
        ::"r"(saddr(dst)), "l"(reinterpret_cast<uint64_t>(m)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(saddr(b))
        : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tmem_alloc(uint32_t* slot, uint32_t cols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(saddr(slot)), "r"(cols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_free(uint32_t taddr, uint32_t cols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(cols) : "memory");
}
// D[tmem] (+)= A[smem] * B[smem]^T, BF16 in, FP32 accumulate.
__device__ __forceinline__ void mma_bf16(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d),
        "l"(a), "l"(b), "r"(idesc), "r"(acc)
        : "memory");
}
// Arrive on b once every MMA this thread issued so far has completed.
__device__ __forceinline__ void mma_commit(uint64_t* b) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(saddr(b))
                 : "memory");
}
// 16 consecutive FP32 columns of this thread's tensor-memory lane.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float v[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int k = 0; k < 16; ++k) v[k] = __uint_as_float(r[k]);
}

// Shared-memory matrix descriptor of a K-major tile whose rows are ROWB bytes
// (32, 64 or 128), swizzled with the matching mode: start address, stride
// between 8-row groups (8 * ROWB), descriptor version 1, layout type.
template <int ROWB>
__device__ __forceinline__ uint64_t sdesc(uint32_t addr) {
    constexpr uint64_t layout = ROWB == 128 ? 2ull : (ROWB == 64 ? 4ull : 6ull);
    return (uint64_t)((addr & 0x3FFFFu) >> 4) | ((uint64_t)1 << 16) | ((uint64_t)((8 * ROWB) >> 4) << 32) |
           ((uint64_t)1 << 46) | (layout << 61);
}
// Instruction descriptor, kind::f16: FP32 accumulator, BF16 A and B, both
// K-major, M = 128, N given.
__host__ __device__ constexpr uint32_t idesc_bf16(int n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(BM >> 4) << 24);
}

__device__ __forceinline__ uint8_t* align1024(uint8_t* p) {
    const uint32_t a = saddr(p);
    return p + ((1024u - (a & 1023u)) & 1023u);
}

template <int COUT, int KC>
struct ConvCfg {
    static constexpr int ROWB = KC * 2;
    static constexpr int A_BYTES = BM * ROWB;
    static constexpr int B_BYTES = COUT * ROWB;
    static constexpr int STAGE = A_BYTES + B_BYTES;
    static constexpr uint32_t TCOLS = COUT < 32 ? 32 : COUT;
    static constexpr int SMEM = 1024 + NST * STAGE + 256;
};

template <int COUT, int KC>
__global__ void __launch_bounds__(128) conv3_kernel(const __grid_constant__ CUtensorMap xmap,
                                                    const __grid_constant__ CUtensorMap wmap, Conv3Args p) {
    using C = ConvCfg<COUT, KC>;
    extern __shared__ uint8_t smem_raw[];
    uint8_t* smem = align1024(smem_raw);
    uint64_t* full = reinterpret_cast<uint64_t*>(smem + NST * C::STAGE);
    uint64_t* empty = full + NST;
    uint64_t* accb = empty + NST;
    uint32_t* tslot = reinterpret_cast<uint32_t*>(accb + 1);
    volatile int* abort_flag = reinterpret_cast<volatile int*>(tslot + 1);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t m0 = (int64_t)blockIdx.x * BM;
    const int64_t hw = (int64_t)p.H * p.W;
    const int z = (int)(m0 / hw);
    const int rem = (int)(m0 % hw);
    const int y0 = rem / p.W, x0 = rem % p.W;
    const int nchunk = p.cin / KC;
    const int steps = 27 * nchunk;

    if (threadIdx.x == 0) {
        for (int s = 0; s < NST; ++s) { bar_init(&full[s], 1); bar_init(&empty[s], 1); }
        bar_init(accb, 1);
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 2) tmem_alloc(tslot, C::TCOLS);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tslot;

    int issued = 0;
    if (warp == 0 && lane == 0) {                       // TMA producer
        for (int s = 0; s < steps; ++s) {
            const int st = s % NST;
            if (s >= NST && !bar_wait(&empty[st], (uint32_t)((s / NST - 1) & 1), abort_flag, p.err, 1)) break;
            const int t = s / nchunk, c = s % nchunk;
            const int dz = t / 9 - 1, dy = (t / 3) % 3 - 1, dx = t % 3 - 1;
            uint8_t* a = smem + st * C::STAGE;
            bar_expect(&full[st], C::STAGE);
            tma4(a, &xmap, &full[st], c * KC, x0 + dx, y0 + dy, z + dz);
            tma3(a + C::A_BYTES, &wmap, &full[st], c * KC, 0, t);
            issued = s + 1;
        }
    } else if (warp == 1 && lane == 0) {                // MMA issuer
        constexpr uint32_t idesc = idesc_bf16(COUT);
        for (int s = 0; s < steps; ++s) {
            const int st = s % NST;
            if (!bar_wait(&full[st], (uint32_t)((s / NST) & 1), abort_flag, p.err, 2)) break;
            tc_fence_after();
            const uint32_t a = saddr(smem + st * C::STAGE);
            const uint32_t b = a + C::A_BYTES;
#pragma unroll
            for (int k = 0; k < KC / 16; ++k)
                mma_bf16(tmem, sdesc<C::ROWB>(a + 32 * k), sdesc<C::ROWB>(b + 32 * k), idesc, (s | k) != 0);
            mma_commit(&empty[st]);
        }
        mma_commit(accb);                               // also fires if nothing was issued
    }
    bool ok = bar_wait(accb, 0, abort_flag, p.err, 3);
    tc_fence_after();
    ok = __syncthreads_and(ok && *abort_flag == 0);
    if (ok) {
        const int row = warp * 32 + lane;
        const int64_t m = m0 + row;
#pragma unroll
        for (int c0 = 0; c0 < COUT; c0 += 16) {
            float v[16];
            tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
            if (p.bias) {
#pragma unroll
                for (int k = 0; k < 16; ++k) v[k] += __ldg(p.bias + c0 + k);
            }
            if (p.act == 1) {
#pragma unroll
                for (int k = 0; k < 16; ++k) v[k] = fmaxf(v[k], 0.0f);
            }
            if (p.mask) {
                const uint4* mk = reinterpret_cast<const uint4*>(p.mask + m * COUT + c0);
                const uint4 u0 = __ldg(mk), u1 = __ldg(mk + 1);
                const uint32_t w[8] = {u0.x, u0.y, u0.z, u0.w, u1.x, u1.y, u1.z, u1.w};
#pragma unroll
                for (int k = 0; k < 8; ++k) {
                    const __nv_bfloat162 h = *reinterpret_cast<const __nv_bfloat162*>(&w[k]);
                    if (!(__bfloat162float(h.x) > 0.0f)) v[2 * k] = 0.0f;
                    if (!(__bfloat162float(h.y) > 0.0f)) v[2 * k + 1] = 0.0f;
                }
            }
            if (p.out_f32) {
                float4* o = reinterpret_cast<float4*>(static_cast<float*>(p.out) + m * COUT + c0);
#pragma unroll
                for (int k = 0; k < 4; ++k) o[k] = make_float4(v[4 * k], v[4 * k + 1], v[4 * k + 2], v[4 * k + 3]);
            } else {
                uint32_t w[8];
#pragma unroll
                for (int k = 0; k < 8; ++k) {
                    const __nv_bfloat162 h = __floats2bfloat162_rn(v[2 * k], v[2 * k + 1]);
                    w[k] = *reinterpret_cast<const uint32_t*>(&h);
                }
                uint4* o = reinterpret_cast<uint4*>(static_cast<__nv_bfloat16*>(p.out) + m * COUT + c0);
                o[0] = make_uint4(w[0], w[1], w[2], w[3]);
                o[1] = make_uint4(w[4], w[5], w[6], w[7]);
            }
        }
    } else if (warp == 0 && lane == 0) {
        // Drain the copies that may still be in flight before shared memory goes away.
        for (int s = issued - NST > 0 ? issued - NST : 0; s < issued; ++s)
            bar_drain(&full[s % NST], (uint32_t)((s / NST) & 1));
    }
    if (!ok && warp == 1 && lane == 0) bar_drain(accb, 0);
    tc_fence_before();
    __syncthreads();
    if (warp == 2) tmem_free(tmem, C::TCOLS);
}

// ---------------------------------------------------------------------------
// Forward convolution over rows of 128 voxels: persistent, with row reuse.
//
// A tile is 128 x-consecutive voxels of one row (W a multiple of 128). Its
// 27 taps read nine input rows -- (dz, dy) in {-1, 0, 1}^2, each 130 voxels
// wide with the x halo. A slice is the three rows (dz = -1, 0, 1) of one y;
// tile y reads slices y - 1, y, y + 1. Tiles are ordered y fastest and dealt
// to the CTAs in groups of RG consecutive tiles, round robin, so the CTAs
// work on neighbouring rows at any moment (each input row is fetched from
// DRAM about once and its other reads hit L2), and inside a group
// consecutive tiles share two of their three slices: a ring of slices in
// shared memory is loaded once each, and a group of RG tiles costs RG + 2
// slices instead of 3 RG. A row is copied
// one 8-channel chunk per copy, so it lands as 130 consecutive 16-byte rows:
// the K-major layout without swizzle (core matrices of 8 rows x 16 bytes,
// 8-row groups 128 bytes apart, channel chunks one padded row block apart),
// and the three x taps of a row start 0, 16 and 32 bytes into it. All 27
// taps' weights stay in shared memory for the CTA's life. Roles: one TMA
// producer thread, one MMA thread issuing the tile's 27 x (cin / 16)
// tcgen05.mma into one of four tensor-memory accumulators, and four epilogue
// warps draining the others (bias, ReLU, mask, conversion, store; an
// accumulator is handed back as soon as it is read, before the stores), so
// the epilogues of earlier tiles overlap the MMAs of later ones.
//
// Shared memory past the slices and the weights keeps spare room, so that
// every descriptor's reach stays inside the allocation whichever way its two
// strides are read.
// ---------------------------------------------------------------------------
constexpr int RCH = 2176;               // one 8-channel chunk of a 130-voxel row (2,080 B), padded to 128 B
constexpr uint32_t RCH_TX = 2080;       // bytes one such copy delivers

template <int COUT, int CIN>
struct RowCfg {
    static constexpr int Q = CIN / 8;                       // 16-byte channel chunks
    static constexpr int RB = Q * RCH;                      // one input row
    static constexpr int SL = 3 * RB;                       // one slice: the rows dz = -1, 0, 1 of one y
    static constexpr int NSL = CIN == 16 ? 12 : 6;          // slices in the ring
    static constexpr int WB = 27 * Q * COUT * 16;           // every tap's weights
    static constexpr int NACC = 4;                          // tensor-memory accumulators
    static constexpr uint32_t TCOLS = NACC * COUT <= 32 ? 32 : (NACC * COUT <= 64 ? 64 : (NACC * COUT <= 128 ? 128 : 256));
    // Farthest byte an A descriptor could address with its two strides
    // exchanged (16 row groups one chunk apart); B's exchanged reach past the
    // weights is under 8 KB.
    static constexpr int REACH = (NSL - 1) * SL + 2 * RB + (Q - 2) * RCH + 48 + 16 * RCH + 256;
    static constexpr int SPARE = REACH - (NSL * SL + WB) > 8192 ? REACH - (NSL * SL + WB) : 8192;
    static constexpr int SMEM = 1024 + NSL * SL + WB + SPARE + 768;
    static constexpr uint32_t TX = 3 * Q * RCH_TX;          // bytes a slice's copies deliver
};

// K-major operand without swizzle: 8-row groups `sbo` bytes apart, 16-byte
// K chunks `lbo` bytes apart.
__device__ __forceinline__ uint64_t sdesc_plain(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((addr & 0x3FFFFu) >> 4) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | ((uint64_t)1 << 46);
}
__device__ __forceinline__ void bar_arrive(uint64_t* b) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(saddr(b)) : "memory");
}

// Tiles y fastest: tile t is (x0, y, z) = ((t / H) % xt * 128, t % H, t / (H * xt)).
// CTA b's i-th tile is t = (b + (i / RG) * gridDim.x) * RG + i % RG.
constexpr int RG = 4;
struct RowTile {
    int x0, y, z;
};
// Tile counts stay below 2^31 (the launcher checks), so the tile arithmetic is 32-bit.
__device__ __forceinline__ RowTile row_tile(int t, int H, int xt) {
    const int r = t / H;
    return RowTile{(r % xt) * BM, t % H, r / xt};
}
__device__ __forceinline__ int row_tile_index(int i) {
    return ((int)blockIdx.x + (i / RG) * (int)gridDim.x) * RG + i % RG;
}
// Whether the CTA's i-th tile t starts a run (its y - 1 and y slices are not
// the previous tile's).
__device__ __forceinline__ bool run_start(int i, int t, int H) {
    return i % RG == 0 || t % H == 0;
}
// Tiles of this CTA: whole groups, less the missing tail of the last group.
__device__ __forceinline__ int row_tiles_of_cta(int ntiles) {
    const int groups = (ntiles + RG - 1) / RG;
    if ((int)blockIdx.x >= groups) return 0;
    const int mine = (groups - 1 - (int)blockIdx.x) / (int)gridDim.x + 1;
    int n = mine * RG;
    if ((int)blockIdx.x + (mine - 1) * (int)gridDim.x == groups - 1) n -= groups * RG - ntiles;
    return n;
}

template <int COUT, int CIN>
__global__ void __launch_bounds__(192, 1) conv3_rows_kernel(const __grid_constant__ CUtensorMap xmap,
                                                            const __nv_bfloat16* __restrict__ wgt, Conv3Args p) {
    using C = RowCfg<COUT, CIN>;
    extern __shared__ uint8_t smem_raw[];
    uint8_t* smem = align1024(smem_raw);
    uint8_t* wsm = smem + C::NSL * C::SL;
    uint64_t* sfull = reinterpret_cast<uint64_t*>(wsm + C::WB + C::SPARE);
    uint64_t* sempty = sfull + C::NSL;
    uint64_t* accf = sempty + C::NSL;
    uint64_t* acce = accf + C::NACC;
    uint32_t* tslot = reinterpret_cast<uint32_t*>(acce + C::NACC);
    volatile int* abort_flag = reinterpret_cast<volatile int*>(tslot + 1);
    float* bias_sm = reinterpret_cast<float*>(tslot + 4);           // COUT floats
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int xt = p.W / BM;
    const int ntiles = p.D * p.H * xt;
    const int my = row_tiles_of_cta(ntiles);

    // Every tap's weights, [tap][chunk][cout][8 channels], written by all
    // threads; the proxy fence makes them visible to the tensor core.
    for (int c = threadIdx.x; c < 27 * C::Q * COUT; c += blockDim.x) {
        const int q = c % C::Q, co = (c / C::Q) % COUT, tap = c / (C::Q * COUT);
        const uint4 v = *reinterpret_cast<const uint4*>(wgt + ((size_t)(tap * COUT + co) * CIN + q * 8));
        *reinterpret_cast<uint4*>(wsm + ((size_t)(tap * C::Q + q) * COUT + co) * 16) = v;
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    for (int c = threadIdx.x; c < COUT; c += blockDim.x) bias_sm[c] = p.bias ? p.bias[c] : 0.0f;
    if (threadIdx.x == 0) {
        for (int s = 0; s < C::NSL; ++s) { bar_init(&sfull[s], 1); bar_init(&sempty[s], 1); }
        for (int a = 0; a < C::NACC; ++a) { bar_init(&accf[a], 1); bar_init(&acce[a], 4); }
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) tmem_alloc(tslot, C::TCOLS);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tslot;

    int loaded = 0, committed = 0;
    if (warp == 0) {
        if (lane == 0) {                                 // TMA producer: slices in order
            bool ok = true;
            for (int i = 0; i < my && ok; ++i) {
                const int t = row_tile_index(i);
                const RowTile c = row_tile(t, p.H, xt);
                const int first = run_start(i, t, p.H) ? -1 : 1;     // y offsets of the new slices
                for (int d = first; d <= 1; ++d) {
                    const int k = loaded, slot = k % C::NSL;
                    if (k >= C::NSL && !bar_wait(&sempty[slot], (uint32_t)((k / C::NSL - 1) & 1), abort_flag, p.err, 11)) {
                        ok = false;
                        break;
                    }
                    uint8_t* sl = smem + slot * C::SL;
                    bar_expect(&sfull[slot], C::TX);
                    for (int dz = 0; dz < 3; ++dz)
#pragma unroll
                        for (int q = 0; q < C::Q; ++q)
                            tma4(sl + dz * C::RB + q * RCH, &xmap, &sfull[slot], q * 8, c.x0 - 1, c.y + d, c.z + dz - 1);
                    loaded = k + 1;
                }
            }
        }
    } else if (warp == 1) {
        if (lane == 0) {                                 // MMA issuer
            constexpr uint32_t idesc = idesc_bf16(COUT);
            // Descriptors are built once; a tap adds its constant offset (in
            // 16-byte units) to the start-address field, which stays below
            // 2^14 for any shared-memory address, so the sum never carries.
            const uint64_t bbase = sdesc_plain(saddr(wsm), COUT * 16, 128);
            int hi = -1;                                 // slice index of the tile's y + 1 row
            for (int i = 0; i < my; ++i) {
                const int t = row_tile_index(i);
                hi += run_start(i, t, p.H) ? 3 : 1;
                const int a = i % C::NACC;
                bool ok = true;
                for (int k = hi - 2; k <= hi && ok; ++k)
                    ok = bar_wait(&sfull[k % C::NSL], (uint32_t)((k / C::NSL) & 1), abort_flag, p.err, 12);
                if (!ok) break;
                if (i >= C::NACC && !bar_wait(&acce[a], (uint32_t)((i / C::NACC - 1) & 1), abort_flag, p.err, 13)) break;
                tc_fence_after();
                const uint32_t d = tmem + (uint32_t)(a * COUT);
                uint64_t abase[3];                       // slices hi - 2, hi - 1, hi (dy = -1, 0, 1)
#pragma unroll
                for (int q = 0; q < 3; ++q)
                    abase[q] = sdesc_plain(saddr(smem + ((hi - 2 + q) % C::NSL) * C::SL), RCH, 128);
#pragma unroll
                for (int tap = 0; tap < 27; ++tap) {
                    // tap = (dz+1)*9 + (dy+1)*3 + (dx+1): slice dy+1, row dz+1, x shift dx+1 rows
#pragma unroll
                    for (int j = 0; j < C::Q / 2; ++j) {
                        const uint64_t ad = abase[(tap / 3) % 3] +
                                            (uint64_t)(((tap / 9) * C::RB + 2 * j * RCH + (tap % 3) * 16) >> 4);
                        const uint64_t bd = bbase + (uint64_t)(((tap * C::Q + 2 * j) * COUT * 16) >> 4);
                        mma_bf16(d, ad, bd, idesc, (tap | j) != 0);
                    }
                }
                // Slices the next tile does not read are free once these MMAs are done.
                const int next_lo = i + 1 < my ? hi + (run_start(i + 1, row_tile_index(i + 1), p.H) ? 3 : 1) - 2 : hi + 1;
                for (int k = hi - 2; k < next_lo && k <= hi; ++k) mma_commit(&sempty[k % C::NSL]);
                mma_commit(&accf[a]);
                committed = i + 1;
            }
        }
    } else {                                             // epilogue: warps 2-5, TMEM lanes of sub-partition warp % 4
        const int sub = warp & 3;
        for (int i = 0; i < my; ++i) {
            const int a = i % C::NACC;
            const bool ok = bar_wait(&accf[a], (uint32_t)((i / C::NACC) & 1), abort_flag, p.err, 14);
            if (!__all_sync(0xFFFFFFFFu, ok)) break;
            tc_fence_after();
            const RowTile c = row_tile(row_tile_index(i), p.H, xt);
            const int64_t m = ((int64_t)c.z * p.H + c.y) * p.W + c.x0 + sub * 32 + lane;
#pragma unroll
            for (int c0 = 0; c0 < COUT; c0 += 16) {
                float v[16];
                tmem_ld16(tmem + ((uint32_t)(sub * 32) << 16) + (uint32_t)(a * COUT + c0), v);
#pragma unroll
                for (int k = 0; k < 16; ++k) v[k] += bias_sm[c0 + k];
                if (p.act == 1) {
#pragma unroll
                    for (int k = 0; k < 16; ++k) v[k] = fmaxf(v[k], 0.0f);
                }
                if (p.mask) {
                    const uint4* mk = reinterpret_cast<const uint4*>(p.mask + m * COUT + c0);
                    const uint4 u0 = __ldg(mk), u1 = __ldg(mk + 1);
                    const uint32_t w[8] = {u0.x, u0.y, u0.z, u0.w, u1.x, u1.y, u1.z, u1.w};
#pragma unroll
                    for (int k = 0; k < 8; ++k) {
                        const __nv_bfloat162 h = *reinterpret_cast<const __nv_bfloat162*>(&w[k]);
                        if (!(__bfloat162float(h.x) > 0.0f)) v[2 * k] = 0.0f;
                        if (!(__bfloat162float(h.y) > 0.0f)) v[2 * k + 1] = 0.0f;
                    }
                }
                if (c0 + 16 >= COUT) {
                    // The accumulator is read out: hand it back before the stores.
                    tc_fence_before();
                    __syncwarp();
                    if (lane == 0) bar_arrive(&acce[a]);
                }
                if (p.out_f32) {
                    float4* o = reinterpret_cast<float4*>(static_cast<float*>(p.out) + m * COUT + c0);
#pragma unroll
                    for (int k = 0; k < 4; ++k) o[k] = make_float4(v[4 * k], v[4 * k + 1], v[4 * k + 2], v[4 * k + 3]);
                } else {
                    uint32_t w[8];
#pragma unroll
                    for (int k = 0; k < 8; ++k) {
                        const __nv_bfloat162 h = __floats2bfloat162_rn(v[2 * k], v[2 * k + 1]);
                        w[k] = *reinterpret_cast<const uint32_t*>(&h);
                    }
                    uint4* o = reinterpret_cast<uint4*>(static_cast<__nv_bfloat16*>(p.out) + m * COUT + c0);
                    o[0] = make_uint4(w[0], w[1], w[2], w[3]);
                    o[1] = make_uint4(w[4], w[5], w[6], w[7]);
                }
            }
        }
    }
    // On an abort, wait (bounded) for this CTA's own copies and MMAs in flight
    // before its shared and tensor memory go away.
    if (*abort_flag) {
        if (warp == 0 && lane == 0)
            for (int k = loaded - C::NSL > 0 ? loaded - C::NSL : 0; k < loaded; ++k)
                bar_drain(&sfull[k % C::NSL], (uint32_t)((k / C::NSL) & 1));
        if (warp == 1 && lane == 0 && committed > 0)
            bar_drain(&accf[(committed - 1) % C::NACC], (uint32_t)(((committed - 1) / C::NACC) & 1));
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 1) tmem_free(tmem, C::TCOLS);
}

template <int CIN, int KV>
struct WgradCfg {
    static constexpr int ROWB = KV * 2;
    static constexpr int A_BYTES = BM * ROWB;        // 128 output-channel rows (beyond Cout: zero fill)
    static constexpr int B_BYTES = CIN * ROWB;
    static constexpr int STAGE = A_BYTES + B_BYTES;
    static constexpr uint32_t TCOLS = CIN < 32 ? 32 : CIN;
    static constexpr int SMEM = 1024 + NST * STAGE + 256;
};

// grid (splits, 27): CTA (s, t) reduces rows [s * rows_per, ...) of tap t.
template <int CIN, int KV>
__global__ void __launch_bounds__(128) wgrad_kernel(const __grid_constant__ CUtensorMap dymap,
                                                    const __grid_constant__ CUtensorMap xmap, WgradArgs p) {
    using C = WgradCfg<CIN, KV>;
    extern __shared__ uint8_t smem_raw[];
    uint8_t* smem = align1024(smem_raw);
    uint64_t* full = reinterpret_cast<uint64_t*>(smem + NST * C::STAGE);
    uint64_t* empty = full + NST;
    uint64_t* accb = empty + NST;
    uint32_t* tslot = reinterpret_cast<uint32_t*>(accb + 1);
    volatile int* abort_flag = reinterpret_cast<volatile int*>(tslot + 1);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int t = blockIdx.y;
    const int dz = t / 9 - 1, dy = (t / 3) % 3 - 1, dx = t % 3 - 1;
    const int rows = p.D * p.H;
    const int r0 = blockIdx.x * p.rows_per_split;
    const int r1 = r0 + p.rows_per_split < rows ? r0 + p.rows_per_split : rows;
    const int xchunks = p.W / KV;
    const int steps = (r1 > r0 ? r1 - r0 : 0) * xchunks;

    if (threadIdx.x == 0) {
        for (int s = 0; s < NST; ++s) { bar_init(&full[s], 1); bar_init(&empty[s], 1); }
        bar_init(accb, 1);
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 2) tmem_alloc(tslot, C::TCOLS);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tslot;

    int issued = 0;
    if (warp == 0 && lane == 0) {
        for (int s = 0; s < steps; ++s) {
            const int st = s % NST;
            if (s >= NST && !bar_wait(&empty[st], (uint32_t)((s / NST - 1) & 1), abort_flag, p.err, 1)) break;
            const int r = r0 + s / xchunks, xc = (s % xchunks) * KV;
            const int z = r / p.H, y = r % p.H;
            uint8_t* a = smem + st * C::STAGE;
            bar_expect(&full[st], C::STAGE);
            tma4(a, &dymap, &full[st], xc, y, z, 0);
            tma4(a + C::A_BYTES, &xmap, &full[st], xc, y + dy, z + dz, (dx + 1) * CIN);
            issued = s + 1;
        }
    } else if (warp == 1 && lane == 0) {
        constexpr uint32_t idesc = idesc_bf16(CIN);
        for (int s = 0; s < steps; ++s) {
            const int st = s % NST;
            if (!bar_wait(&full[st], (uint32_t)((s / NST) & 1), abort_flag, p.err, 2)) break;
            tc_fence_after();
            const uint32_t a = saddr(smem + st * C::STAGE);
            const uint32_t b = a + C::A_BYTES;
#pragma unroll
            for (int k = 0; k < KV / 16; ++k)
                mma_bf16(tmem, sdesc<C::ROWB>(a + 32 * k), sdesc<C::ROWB>(b + 32 * k), idesc, (s | k) != 0);
            mma_commit(&empty[st]);
        }
        mma_commit(accb);
    }
    bool ok = bar_wait(accb, 0, abort_flag, p.err, 3);
    tc_fence_after();
    ok = __syncthreads_and(ok && *abort_flag == 0);
    if (ok) {
        const int co = warp * 32 + lane;
        float* dst = p.partial + ((int64_t)t * gridDim.x + blockIdx.x) * p.cout * CIN;
#pragma unroll
        for (int c0 = 0; c0 < CIN; c0 += 16) {
            float v[16];
            tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
            if (steps == 0) {
#pragma unroll
                for (int k = 0; k < 16; ++k) v[k] = 0.0f;
            }
            if (co < p.cout) {
                float4* o = reinterpret_cast<float4*>(dst + (int64_t)co * CIN + c0);
#pragma unroll
                for (int k = 0; k < 4; ++k) o[k] = make_float4(v[4 * k], v[4 * k + 1], v[4 * k + 2], v[4 * k + 3]);
            }
        }
    } else if (warp == 0 && lane == 0) {
        for (int s = issued - NST > 0 ? issued - NST : 0; s < issued; ++s)
            bar_drain(&full[s % NST], (uint32_t)((s / NST) & 1));
    }
    if (!ok && warp == 1 && lane == 0) bar_drain(accb, 0);
    tc_fence_before();
    __syncthreads();
    if (warp == 2) tmem_free(tmem, C::TCOLS);
}

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
using Encode = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                            const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                            CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
Encode encoder() {
    static Encode enc = nullptr;
    if (!enc) {
        void* fn = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            enc = reinterpret_cast<Encode>(fn);
    }
    return enc;
}

CUtensorMapSwizzle swizzle_for(int rowb) {
    return rowb == 128 ? CU_TENSOR_MAP_SWIZZLE_128B : (rowb == 64 ? CU_TENSOR_MAP_SWIZZLE_64B : CU_TENSOR_MAP_SWIZZLE_32B);
}

// rowb 0: no swizzle (the row kernel's copies); otherwise the swizzle matching a rowb-byte row.
bool map_bf16(CUtensorMap* m, const void* base, int rank, const uint64_t* dims, const uint32_t* box, int rowb) {
    Encode enc = encoder();
    if (!enc) return false;
    cuuint64_t d[5], st[4];
    cuuint32_t b[5], es[5];
    uint64_t stride = 2;
    for (int i = 0; i < rank; ++i) {
        d[i] = dims[i];
        b[i] = box[i];
        es[i] = 1;
        if (i > 0) st[i - 1] = stride;
        stride *= dims[i];
    }
    return enc(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, (cuuint32_t)rank, const_cast<void*>(base), d, st, b, es,
               CU_TENSOR_MAP_INTERLEAVE_NONE, rowb == 0 ? CU_TENSOR_MAP_SWIZZLE_NONE : swizzle_for(rowb),
               CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

template <int COUT, int KC>
cudaError_t launch_conv(const Conv3Args& a, const void* x, const void* w, cudaStream_t s) {
    using C = ConvCfg<COUT, KC>;
    CUtensorMap xm, wm;
    const uint64_t xd[4] = {(uint64_t)a.cin, (uint64_t)a.W, (uint64_t)a.H, (uint64_t)a.D};
    const uint32_t xb[4] = {(uint32_t)KC, (uint32_t)(a.W < BM ? a.W : BM), (uint32_t)(a.W < BM ? BM / a.W : 1), 1};
    const uint64_t wd[3] = {(uint64_t)a.cin, (uint64_t)COUT, 27};
    const uint32_t wb[3] = {(uint32_t)KC, (uint32_t)COUT, 1};
    if (!map_bf16(&xm, x, 4, xd, xb, C::ROWB) || !map_bf16(&wm, w, 3, wd, wb, C::ROWB))
        return cudaErrorInvalidValue;
    static bool attr = false;
    if (!attr) {
        cudaFuncSetAttribute(conv3_kernel<COUT, KC>, cudaFuncAttributeMaxDynamicSharedMemorySize, C::SMEM);
        attr = true;
    }
    const int64_t m = (int64_t)a.D * a.H * a.W;
    conv3_kernel<COUT, KC><<<(unsigned)(m / BM), 128, C::SMEM, s>>>(xm, wm, a);
    return cudaGetLastError();
}

int sm_count() {
    static int n = 0;
    if (n == 0) {
        int d = 0;
        cudaGetDevice(&d);
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, d);
        if (n <= 0) n = 1;
    }
    return n;
}

template <int COUT, int CIN>
cudaError_t launch_conv_rows(const Conv3Args& a, const void* x, const void* w, cudaStream_t s) {
    using C = RowCfg<COUT, CIN>;
    static_assert(C::SMEM <= 232448, "row kernel shared memory");
    CUtensorMap xm;
    const uint64_t xd[4] = {(uint64_t)a.cin, (uint64_t)a.W, (uint64_t)a.H, (uint64_t)a.D};
    const uint32_t xb[4] = {8u, (uint32_t)(BM + 2), 1u, 1u};
    if (!map_bf16(&xm, x, 4, xd, xb, 0)) return cudaErrorInvalidValue;
    static bool attr = false;
    if (!attr) {
        cudaFuncSetAttribute(conv3_rows_kernel<COUT, CIN>, cudaFuncAttributeMaxDynamicSharedMemorySize, C::SMEM);
        attr = true;
    }
    const int64_t tiles = (int64_t)a.D * a.H * (a.W / BM);
    if (tiles >= (1LL << 31) - RG) return cudaErrorInvalidValue;
    const int sms = sm_count();
    const int64_t groups = (tiles + RG - 1) / RG;
    const unsigned grid = (unsigned)(groups < sms ? groups : sms);    // one CTA per SM
    conv3_rows_kernel<COUT, CIN><<<grid, 192, C::SMEM, s>>>(xm, static_cast<const __nv_bfloat16*>(w), a);
    return cudaGetLastError();
}

template <int CIN, int KV>
cudaError_t launch_wgrad(const WgradArgs& a, const void* dyt, const void* xt3, cudaStream_t s) {
    using C = WgradCfg<CIN, KV>;
    CUtensorMap dm, xm;
    const uint64_t dd[4] = {(uint64_t)a.W, (uint64_t)a.H, (uint64_t)a.D, (uint64_t)a.cout};
    const uint32_t db[4] = {(uint32_t)KV, 1, 1, (uint32_t)BM};
    const uint64_t xd[4] = {(uint64_t)a.W, (uint64_t)a.H, (uint64_t)a.D, (uint64_t)(3 * CIN)};
    const uint32_t xb[4] = {(uint32_t)KV, 1, 1, (uint32_t)CIN};
    if (!map_bf16(&dm, dyt, 4, dd, db, C::ROWB) || !map_bf16(&xm, xt3, 4, xd, xb, C::ROWB))
        return cudaErrorInvalidValue;
    static bool attr = false;
    if (!attr) {
        cudaFuncSetAttribute(wgrad_kernel<CIN, KV>, cudaFuncAttributeMaxDynamicSharedMemorySize, C::SMEM);
        attr = true;
    }
    wgrad_kernel<CIN, KV><<<dim3((unsigned)a.splits, 27), 128, C::SMEM, s>>>(dm, xm, a);
    return cudaGetLastError();
}

}  // namespace

bool conv3_supported(int D, int H, int W, int cin, int cout) {
    const bool wok = W == 32 || W == 64 || (W % 128 == 0 && W <= 256);
    const bool cok = (cin == 16 || cin == 32 || cin % 64 == 0) && cin <= 256 &&
                     (cout == 16 || cout == 32 || cout == 64 || cout == 128);
    return D > 0 && H > 0 && wok && ((int64_t)H * W) % BM == 0 && cok;
}

cudaError_t conv3(const Conv3Args& a, const void* x, const void* w, cudaStream_t s) {
    if (!conv3_supported(a.D, a.H, a.W, a.cin, a.cout)) return cudaErrorInvalidValue;
    // Rows of 128 voxels with 16 or 32 input channels: the persistent row kernel.
    if (a.W % BM == 0) {
#define AGB_ROW_CASE(CO, CI) \
        if (a.cout == CO && a.cin == CI) return launch_conv_rows<CO, CI>(a, x, w, s);
        AGB_ROW_CASE(16, 16) AGB_ROW_CASE(32, 16) AGB_ROW_CASE(64, 16)
        AGB_ROW_CASE(16, 32) AGB_ROW_CASE(32, 32)
#undef AGB_ROW_CASE
    }
    const int kc = a.cin >= 64 ? 64 : a.cin;
#define AGB_CONV_CASE(CO, K) \
    if (a.cout == CO && kc == K) return launch_conv<CO, K>(a, x, w, s);
    AGB_CONV_CASE(16, 16) AGB_CONV_CASE(16, 32) AGB_CONV_CASE(16, 64)
    AGB_CONV_CASE(32, 16) AGB_CONV_CASE(32, 32) AGB_CONV_CASE(32, 64)
    AGB_CONV_CASE(64, 16) AGB_CONV_CASE(64, 32) AGB_CONV_CASE(64, 64)
    AGB_CONV_CASE(128, 16) AGB_CONV_CASE(128, 32) AGB_CONV_CASE(128, 64)
#undef AGB_CONV_CASE
    return cudaErrorInvalidValue;
}

bool wgrad_supported(int D, int H, int W, int cin, int cout) {
    return D > 0 && H > 0 && (W == 32 || W % 64 == 0) && (cin == 16 || cin == 32 || cin == 64 || cin == 128) &&
           cout >= 1 && cout <= BM;
}

cudaError_t wgrad(const WgradArgs& a, const void* dyt, const void* xt3, cudaStream_t s) {
    if (!wgrad_supported(a.D, a.H, a.W, a.cin, a.cout) || a.splits <= 0 || a.rows_per_split <= 0)
        return cudaErrorInvalidValue;
    const int kv = a.W >= 64 ? 64 : a.W;
#define AGB_WG_CASE(CI, K) \
    if (a.cin == CI && kv == K) return launch_wgrad<CI, K>(a, dyt, xt3, s);
    AGB_WG_CASE(16, 32) AGB_WG_CASE(16, 64) AGB_WG_CASE(32, 32) AGB_WG_CASE(32, 64)
    AGB_WG_CASE(64, 32) AGB_WG_CASE(64, 64) AGB_WG_CASE(128, 32) AGB_WG_CASE(128, 64)
#undef AGB_WG_CASE
    return cudaErrorInvalidValue;
}

}  // namespace nn
}  // namespace agb
