// Blackwell (sm_100 family) tensor-core GEMM for the warm-start network's
// convolutions: tcgen05.mma with BF16 operands staged in shared memory and
// the FP32 accumulator in tensor memory (TMEM).
//
//   D[M x N] = sum_k A(m, k) B(n, k)      (both operands K-major)
//
// One CTA of 128 threads computes a 128 x NT tile of D (NT = 16 .. 256, a
// multiple of 16) over a range of K (split-K over gridDim.z).  For each
// K-chunk of 64 the 128 threads gather the A tile (128 x 64) and the B tile
// (NT x 64) into shared memory in the canonical no-swizzle K-major layout
// (8 x 16-byte core matrices: rows of a core matrix 16 bytes apart, core
// matrices 128 bytes apart along K and 1024 bytes apart along M / N), make
// the writes visible to the tensor core (fence.proxy.async), and one thread
// issues four 128 x NT x 16 MMAs and commits them to an mbarrier.  kStages
// chunk buffers form a ring: the copies of chunks c+1 .. c+kStages-1 are in
// flight (cp.async, 16 bytes each, zero-filled outside the operand) while
// the MMAs of chunk c run.  The epilogue reads the accumulator with
// tcgen05.ld: warp w owns TMEM lanes (= rows of D) 32w .. 32w + 31.
//
// A loader functor gives the 8 consecutive K elements of one row: an
// asynchronous loader (kAsync = true) their 16-byte-aligned global address
// (src(), null for zeros), a gathering loader (kAsync = false) their value as
// a uint4 (operator(), zeros outside the operand), which the threads store
// into the ring themselves.  The epilogue functor receives (split, m, n,
// value).
#pragma once

#include <cstdint>

#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

namespace rf_tc {

constexpr int kTM = 128;      // rows of D per CTA (the MMA's M)
constexpr int kTK = 64;       // K per chunk (four MMAs of K = 16)
constexpr int kThreads = 128;
// bounded waits: an mbarrier that does not complete in this many polls
// marks the launch as failed (see k_tc_gemm)
constexpr unsigned kSpinLimit = 1u << 26;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// shared-memory matrix descriptor (tcgen05): start address, leading (K)
// and stride (M / N) byte offsets in 16-byte units, descriptor version 1 at
// bit 46, no swizzle (layout type 0 in bits 61..63)
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = 0;
    d |= (uint64_t)((addr >> 4) & 0x3FFFu);
    d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1 << 46;
    return d;
}

// instruction descriptor, kind::f16: D = F32 (bits 4..5 = 1), A = B = BF16
// (bits 7..9 and 10..12 = 1), both K-major (bits 15, 16 = 0), N >> 3 in
// bits 17..22, M >> 4 in bits 24..28
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) |
           ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
                 : "memory");
}

// bounded wait on an mbarrier phase (at most `limit` polls); false if it did
// not complete
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, unsigned parity,
                                          unsigned limit = kSpinLimit) {
    const uint32_t a = smem_u32(bar);
    for (unsigned i = 0; i < limit; i++) {
        uint32_t done;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
            " selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(a), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

__device__ __forceinline__ void fence_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_before() {
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

__device__ __forceinline__ void tmem_alloc(uint32_t* dst_smem, uint32_t ncols) {
    asm volatile(
        "tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n"
        "tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::"r"(smem_u32(dst_smem)),
        "r"(ncols)
        : "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols)
                 : "memory");
}

__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc,
                                         uint32_t accumulate) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.u32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
        "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
        : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t* bar) {
    asm volatile(
        "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
            smem_u32(bar))
        : "memory");
}

// 8 consecutive 32-bit TMEM columns of this thread's lane
__device__ __forceinline__ void tmem_ld8(uint32_t taddr, float (&v)[8]) {
    uint32_t r[8];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];\n"
        "tcgen05.wait::ld.sync.aligned;\n"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
          "=r"(r[7])
        : "r"(taddr)
        : "memory");
#pragma unroll
    for (int i = 0; i < 8; i++) v[i] = __uint_as_float(r[i]);
}

// byte offset of element row r, k-group g (8 elements) in a chunk tile
__device__ __forceinline__ uint32_t tile_off(int r, int g) {
    return (uint32_t)(((r >> 3) * (kTK / 8) + g) * 128 + (r & 7) * 16);
}

__device__ __forceinline__ void cp_async16(void* smem_dst, const void* gsrc, int src_bytes) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(smem_u32(smem_dst)),
                 "l"(gsrc), "r"(src_bytes)
                 : "memory");
}
__device__ __forceinline__ void cp_async_commit() {
    asm volatile("cp.async.commit_group;" ::: "memory");
}
template <int N>
__device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// chunk buffers in the ring: three when a loader copies asynchronously (two
// chunks in flight during an MMA), two when both gather through registers
// (their stores finish before the chunk's barrier anyway; less shared
// memory keeps more CTAs resident)
template <class LA, class LB>
constexpr int stages_for() {
    return (LA::kAsync || LB::kAsync) ? 3 : 2;
}

template <int NT, int kStages>
struct TcSmem {
    static_assert(NT % 16 == 0 && NT >= 16 && NT <= 256, "N tile");
    static_assert((NT * 8) % 128 == 0, "B tile rows split evenly over the CTA's threads");
    static constexpr int kA = kTM * kTK * 2;  // bytes of one A chunk
    static constexpr int kB = NT * kTK * 2;
    // the chunk ring, barriers, alignment slack
    static constexpr int kBytes = kStages * (kA + kB) + 2048;
    static constexpr uint32_t kCols = NT <= 32 ? 32 : (NT <= 64 ? 64 : (NT <= 128 ? 128 : 256));
};

// grid: x = M tiles, y = N tiles, z = K splits (each `kspan` long, a multiple
// of kTK).  `status` (device int) is set to 1 if a wait gave up; the launch's
// outputs are then not written.  A thread whose wait for a ring slot gives up
// writes no further chunks (an MMA may still be reading that slot); the MMA
// thread keeps issuing and committing, and every thread drains the last
// commit with the full limit before TMEM is released, so TMEM is freed under
// MMAs in flight only if that second wait runs out too.  `first_wait_polls`
// >= 0 caps the first slot wait of each CTA at that many polls (a test hook:
// 0 makes it give up at once while the MMAs still complete); -1 = the
// normal limit.
template <int NT, class LA, class LB, class EP>
__global__ void __launch_bounds__(kThreads) k_tc_gemm(int M, int N, int K, int kspan, LA la,
                                                     LB lb, EP ep, int* status,
                                                     int first_wait_polls) {
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    constexpr int kStages = stages_for<LA, LB>();
    using S = TcSmem<NT, kStages>;
    unsigned char* base = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    uint64_t* bars = (uint64_t*)(base + kStages * (S::kA + S::kB));  // one per ring slot
    uint32_t* tslot = (uint32_t*)(bars + kStages);
    int* fail = (int*)(tslot + 1);

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int m0 = blockIdx.x * kTM, n0 = blockIdx.y * NT;
    const int k_begin = blockIdx.z * kspan;
    const int k_end = min(K, k_begin + kspan);
    const int nchunks = (k_end - k_begin + kTK - 1) / kTK;

    if (tid == 0) {
        for (int q = 0; q < kStages; q++) mbar_init(&bars[q], 1);
        *fail = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) tmem_alloc(tslot, S::kCols);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tslot;
    constexpr uint32_t idesc = idesc_bf16(kTM, NT);

    // queue the copies (or do the gathers) of chunk c into ring slot c % kStages
    auto issue = [&](int c) {
        const int q = c % kStages;
        unsigned char* tA = base + q * S::kA;
        unsigned char* tB = base + kStages * S::kA + q * S::kB;
        const int kc = k_begin + c * kTK;
        constexpr int kPerA = kTM * (kTK / 8) / kThreads;  // 8
        constexpr int kPerB = NT * (kTK / 8) / kThreads;   // NT / 16
        if constexpr (LA::kAsync) {
#pragma unroll
            for (int j = 0; j < kPerA; j++) {
                const int i = tid + j * kThreads, r = i >> 3, g = i & 7, k = kc + g * 8;
                const void* src = (m0 + r < M && k < k_end) ? la.src(m0 + r, k) : nullptr;
                cp_async16(tA + tile_off(r, g), src ? src : la.base(), src ? 16 : 0);
            }
        } else {
            // all of a thread's loads are issued before its stores (the stores go
            // through a generic pointer the compiler cannot tell from global memory)
            uint4 va[kPerA];
#pragma unroll
            for (int j = 0; j < kPerA; j++) {
                const int i = tid + j * kThreads, r = i >> 3, g = i & 7, k = kc + g * 8;
                va[j] = make_uint4(0, 0, 0, 0);
                if (m0 + r < M && k < k_end) va[j] = la(m0 + r, k, k_end);
            }
#pragma unroll
            for (int j = 0; j < kPerA; j++) {
                const int i = tid + j * kThreads;
                *(uint4*)(tA + tile_off(i >> 3, i & 7)) = va[j];
            }
        }
        if constexpr (LB::kAsync) {
#pragma unroll
            for (int j = 0; j < kPerB; j++) {
                const int i = tid + j * kThreads, r = i >> 3, g = i & 7, k = kc + g * 8;
                const void* src = (n0 + r < N && k < k_end) ? lb.src(n0 + r, k) : nullptr;
                cp_async16(tB + tile_off(r, g), src ? src : lb.base(), src ? 16 : 0);
            }
        } else {
            uint4 vb[kPerB];
#pragma unroll
            for (int j = 0; j < kPerB; j++) {
                const int i = tid + j * kThreads, r = i >> 3, g = i & 7, k = kc + g * 8;
                vb[j] = make_uint4(0, 0, 0, 0);
                if (n0 + r < N && k < k_end) vb[j] = lb(n0 + r, k, k_end);
            }
#pragma unroll
            for (int j = 0; j < kPerB; j++) {
                const int i = tid + j * kThreads;
                *(uint4*)(tB + tile_off(i >> 3, i & 7)) = vb[j];
            }
        }
    };

    // prologue: chunks 0 .. kStages-2 in flight; one commit group per chunk
    // (empty past the end) keeps the group count uniform
    for (int c = 0; c < kStages - 1; c++) {
        if (c < nchunks) issue(c);
        cp_async_commit();
    }
    bool gave_up = false;  // this thread's slot wait ran out: it writes no more chunks
    for (int c = 0; c < nchunks; c++) {
        const int q = c % kStages;
        cp_async_wait<kStages - 2>();  // chunk c has landed
        fence_async_smem();
        __syncthreads();
        if (tid == 0) {
            tc_fence_after();
            const uint32_t a0 = smem_u32(base + q * S::kA);
            const uint32_t b0 = smem_u32(base + kStages * S::kA + q * S::kB);
#pragma unroll
            for (int kk = 0; kk < kTK / 16; kk++) {
                const uint64_t da = smem_desc(a0 + kk * 256, 128, 1024);
                const uint64_t db = smem_desc(b0 + kk * 256, 128, 1024);
                mma_bf16(tmem, da, db, idesc, (c > 0 || kk > 0) ? 1u : 0u);
            }
            mma_commit(&bars[q]);
        }
        // refill the slot chunk c - 1 used once its MMAs are done
        const int nc = c + kStages - 1;
        if (nc < nchunks && !gave_up) {
            if (c >= 1) {
                const int pc = c - 1;
                const unsigned lim = (c == 1 && first_wait_polls >= 0) ? (unsigned)first_wait_polls
                                                                       : kSpinLimit;
                if (!mbar_wait(&bars[pc % kStages], (unsigned)(pc / kStages) & 1u, lim)) {
                    gave_up = true;
                    *fail = 1;
                }
            }
            if (!gave_up) issue(nc);
        }
        cp_async_commit();
    }
    // the last commit covers every earlier MMA of this CTA
    cp_async_wait<0>();
    if (nchunks > 0) {
        const int lc = nchunks - 1;
        if (!mbar_wait(&bars[lc % kStages], (unsigned)(lc / kStages) & 1u)) *fail = 1;
    }
    tc_fence_after();
    __syncthreads();
    if (*fail) {
        if (tid == 0) atomicExch(status, 1);
    } else if (nchunks > 0) {
        const int m = m0 + warp * 32 + lane;
        const uint32_t lane_addr = tmem + ((uint32_t)(warp * 32) << 16);
#pragma unroll 1
        for (int j = 0; j < NT; j += 8) {
            float v[8];
            tmem_ld8(lane_addr + (uint32_t)j, v);
            if (m < M)
#pragma unroll
                for (int e = 0; e < 8; e++)
                    if (n0 + j + e < N) ep(blockIdx.z, m, n0 + j + e, v[e]);
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) tmem_dealloc(tmem, S::kCols);
}

// ---------------------------------------------------------------------------
// Direct 3x3 convolution (stride 1, padding 1) on padded activations
// ---------------------------------------------------------------------------
// Activations are NHWC with a one-pixel zero border: position
// q = (b (H + 2) + y) (W + 2) + x of a [B][H + 2][W + 2][C] buffer.  For
// output position q, tap (dy, dx) reads input position
// q + (dy - 1)(W + 2) + (dx - 1), so 128 consecutive output positions read
// 128 consecutive input positions for every tap: each tap is one MMA whose
// A operand is a shifted view of one staged slab, and no im2col copy exists.
// A CTA computes positions [q0, q0 + 128) (border positions too; their
// outputs are not stored, so borders stay zero).  Per stage of 16 input
// channels it stages, by TMA, the slab of input positions
// [q0 - (W + 3), q0 + 128 + (W + 3)) as two planes of 8 channels (16 bytes
// per position: the canonical no-swizzle K-major layout, core matrices of 8
// positions, the two K halves one plane apart), and by a bulk copy the
// stage's weights for all 9 taps in the same layout (host-prepared), then
// one thread issues the 9 MMAs (M = 128, N = NT, K = 16) into the TMEM
// accumulator.  kConvStages ring slots: loads of the next stages run while
// a stage's MMAs do.  Out-of-range slab positions (before the first image,
// past the buffer) are filled with zeros by the TMA unit and only reach
// border outputs.
constexpr int kConvBox = 128;  // positions per TMA box (2 KB per 8-channel plane)

struct ConvGeom {
    int Wp;      // padded row length W + 2
    int npos;    // padded positions of this call: B (H + 2)(W + 2)
    int nbox;    // TMA boxes per plane: ceil((128 + 2 (W + 3)) / 128)
    int stages;  // input channels / 16
};

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
                 "r"(bytes)
                 : "memory");
}

// 2D tile of the tensor map at (c0 = channel, c1 = position) into shared memory
__device__ __forceinline__ void tma_load_2d(void* dst, const void* map, int c0, int c1,
                                            uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3}], [%4];" ::"r"(smem_u32(dst)),
        "l"(map), "r"(c0), "r"(c1), "r"(smem_u32(bar))
        : "memory");
}

// contiguous bytes (16-byte aligned, a multiple of 16) into shared memory
__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes,
                                          uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
            "r"(smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}

template <int NT>
struct ConvSmem {
    static_assert(NT % 16 == 0 && NT >= 16 && NT <= 128, "N tile");
    static constexpr int kStages = NT >= 96 ? 2 : 3;
    static constexpr uint32_t kWBytes = 9u * NT * 32u;  // one stage's weights
    static constexpr uint32_t kCols = NT <= 32 ? 32 : (NT <= 64 ? 64 : 128);
    __host__ __device__ static uint32_t plane_bytes(int nbox) { return (uint32_t)nbox * kConvBox * 16u; }
    __host__ __device__ static uint32_t stage_bytes(int nbox) { return 2u * plane_bytes(nbox) + kWBytes; }
    static size_t bytes(int nbox) { return (size_t)kStages * stage_bytes(nbox) + 2048; }
};

// `xmap`: CUtensorMap over the padded input viewed as [positions][C] BF16
// (box: 8 channels x kConvBox positions); `wc`: weights as
// [stage][tap][NT / 8][2][8][8] BF16.  `status` is set to 1 if a wait gave
// up (the launch's outputs are then not written); `first_wait_polls` >= 0
// caps the first slab wait of each CTA (a test hook, as for k_tc_gemm).
// Every load issued is waited for (with the full limit) before the CTA
// ends, and the last MMA commit before TMEM is released.
template <int NT, class EP>
__global__ void __launch_bounds__(kThreads) k_tc_conv3(const __grid_constant__ CUtensorMap xmap,
                                                      const __nv_bfloat16* __restrict__ wc,
                                                      ConvGeom g, EP ep, int* status,
                                                      int first_wait_polls) {
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    using S = ConvSmem<NT>;
    constexpr int kS = S::kStages;
    unsigned char* base = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    const uint32_t plane = S::plane_bytes(g.nbox);
    const uint32_t stage_bytes = S::stage_bytes(g.nbox);
    uint64_t* full = (uint64_t*)(base + kS * stage_bytes);
    uint64_t* empty = full + kS;
    uint32_t* tslot = (uint32_t*)(empty + kS);
    int* fail = (int*)(tslot + 1);
    int* produced = fail + 1;   // stages whose loads were issued
    int* committed = fail + 2;  // stages whose MMAs were committed

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int q0 = blockIdx.x * kTM;
    const int halo = g.Wp + 1;
    const int nst = g.stages;

    if (tid == 0) {
        for (int q = 0; q < kS; q++) {
            mbar_init(&full[q], 1);
            mbar_init(&empty[q], 1);
        }
        *fail = 0;
        *produced = 0;
        *committed = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) tmem_alloc(tslot, S::kCols);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tslot;
    constexpr uint32_t idesc = idesc_bf16(kTM, NT);

    auto produce = [&](int j) {
        const int sl = j % kS;
        unsigned char* st = base + sl * stage_bytes;
        mbar_expect_tx(&full[sl], stage_bytes);
        for (int pl = 0; pl < 2; pl++)
            for (int b = 0; b < g.nbox; b++)
                tma_load_2d(st + pl * plane + b * (kConvBox * 16), &xmap, 16 * j + 8 * pl,
                            q0 - halo + b * kConvBox, &full[sl]);
        bulk_load(st + 2 * plane, wc + (size_t)j * 9 * NT * 16, S::kWBytes, &full[sl]);
        *produced = j + 1;
    };

    if (tid == 0) {
        for (int j = 0; j < kS && j < nst; j++) produce(j);
        for (int j = 0; j < nst; j++) {
            const int sl = j % kS;
            const unsigned lim = (j == 0 && first_wait_polls >= 0) ? (unsigned)first_wait_polls
                                                                  : kSpinLimit;
            if (!mbar_wait(&full[sl], (unsigned)(j / kS) & 1u, lim)) {
                *fail = 1;
                break;
            }
            tc_fence_after();
            const uint32_t a0 = smem_u32(base + sl * stage_bytes);
            const uint32_t b0 = a0 + 2 * plane;
#pragma unroll
            for (int t = 0; t < 9; t++) {
                const int off = halo + (t / 3 - 1) * g.Wp + (t % 3 - 1);
                const uint64_t da = smem_desc(a0 + (uint32_t)off * 16u, plane, 128);
                const uint64_t db = smem_desc(b0 + (uint32_t)t * NT * 32u, 128, 256);
                mma_bf16(tmem, da, db, idesc, (j > 0 || t > 0) ? 1u : 0u);
            }
            mma_commit(&empty[sl]);
            *committed = j + 1;
            // refill the slot of stage j - 1 once its MMAs are done (stage j's
            // MMAs stay queued meanwhile)
            const int pj = j - 1;
            if (pj >= 0 && pj + kS < nst) {
                if (!mbar_wait(&empty[pj % kS], (unsigned)(pj / kS) & 1u)) {
                    *fail = 1;
                    break;
                }
                produce(pj + kS);
            }
        }
    }
    __syncthreads();
    // drain: every load issued has landed and the last commit (which covers
    // every earlier MMA) has arrived, each with the full limit
    if (tid == 0) {
        const int np = *produced, nc = *committed;
        for (int j = nc; j < np; j++)  // loads no MMA waited for
            if (!mbar_wait(&full[j % kS], (unsigned)(j / kS) & 1u)) *fail = 1;
        if (nc > 0 && !mbar_wait(&empty[(nc - 1) % kS], (unsigned)((nc - 1) / kS) & 1u))
            *fail = 1;
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (*fail) {
        if (tid == 0) atomicExch(status, 1);
    } else if (nst > 0) {
        const int q = q0 + warp * 32 + lane;
        const int p = ep.pos(q);  // < 0: a border position or past the call's positions
        const uint32_t lane_addr = tmem + ((uint32_t)(warp * 32) << 16);
#pragma unroll 1
        for (int c = 0; c < NT; c += 8) {
            float v[8];
            tmem_ld8(lane_addr + (uint32_t)c, v);
            if (p >= 0) ep.store(q, p, c, v);
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) tmem_dealloc(tmem, S::kCols);
}

}  // namespace rf_tc
