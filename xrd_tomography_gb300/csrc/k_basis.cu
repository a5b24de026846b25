// k_basis.cu -- basis expansion on the 5th-generation tensor cores:
// I[M x N] = C[M x K] B[K x N] in FP32 through 3xTF32.
//
// The reference's coarse q "basis" is point-sampled (wvt_value.cu:8-22,
// integrate_diffraction.cu:311-315): each coefficient is a Gaussian
// evaluated at one bin centre, a diagonal basis with no contraction.  A dense
// basis -- K coefficients per material or voxel expanded onto N q bins -- is
// the one GEMM-shaped operation of the model.  With K <= 64 it moves 4(K + N)
// bytes per row for 6KN flops, so it is bound by HBM, not by the tensor
// rate; the kernel is built to keep HBM busy:
//
//  * persistent CTAs (4 warps) loop over 128-row tiles of C; the basis is
//    split and staged in shared memory once per CTA, in the canonical
//    K-major layout without swizzle (core matrices of 8 rows x 16 bytes);
//  * FP32 accuracy from TF32 inputs: x = hi + lo with hi, lo rounded to TF32,
//    and D = A_hi B_hi + A_hi B_lo + A_lo B_hi accumulated in FP32 in tensor
//    memory (the dropped A_lo B_lo term is below 2^-22 of the product);
//  * two accumulators in tensor memory: while the MMAs of tile g run, the
//    four warps read tile g-1's accumulator back (tcgen05.ld) and store its
//    rows;
//  * the tiles of C arrive ahead of use: through the bulk-copy engine into a
//    ring of shared-memory stages (one cp.async.bulk per tile, completing on
//    the stage's mbarrier) when C is 16-byte aligned and two stages fit,
//    else as 16-byte loads into registers during the MMAs; either way a warp
//    instruction covers 8 rows x 64 bytes, which keeps the shared-memory
//    stores of the split free of bank conflicts;
//  * one thread issues the MMAs (K = 8 each) and commits each tile's to the
//    mbarrier of its accumulator.
//
// Every mbarrier wait is bounded: on time-out the kernel raises an error
// flag, stops taking tiles, waits (again bounded) for the MMAs it committed
// and still frees its tensor memory.
#include <cstdlib>
#include "xrdt_device.cuh"

namespace xrdt {

namespace {

constexpr int kTileM = 128;
constexpr int kBasisThreads = 128;
constexpr int kMaxK = 64;
constexpr unsigned kSpinLimit = 1u << 26;

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// TF32 rounding (nearest, ties away from zero): the high part of a split.
__device__ __forceinline__ float tf32_rna(float x)
{
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return __uint_as_float(r);
}

// Canonical K-major layout without swizzle: element (r, k) of a tile with K
// columns at byte (r/8)(K/4)128 + (k/4)128 + (r%8)16 + (k%4)4, i.e. core
// matrices of 8 rows x 16 bytes, adjacent in K 128 bytes apart and adjacent
// in rows (K/4)128 bytes apart.
__device__ __forceinline__ int kmajor_offset(int r, int k, int K)
{
    return (r >> 3) * (K >> 2) * 128 + (k >> 2) * 128 + (r & 7) * 16 + (k & 3) * 4;
}

// Shared-memory matrix descriptor: start address, leading byte offset (the
// K-adjacent core matrix), stride byte offset (the next 8 rows), descriptor
// version 1, base offset 0, no swizzle.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo)
{
    uint64_t d = (uint64_t)((addr >> 4) & 0x3FFFu);
    d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1 << 46;
    return d;
}

// Instruction descriptor of kind::tf32: FP32 accumulator, TF32 A and B,
// both K-major, no negation, N/8 and M/16.
__host__ __device__ constexpr uint32_t idesc_tf32(int M, int N)
{
    return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// Bounded wait for phase `parity` of the mbarrier at `bar`; false on time-out.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, unsigned limit)
{
    uint32_t done = 0;
    for (unsigned it = 0; !done; it++) {
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}\n"
            : "=r"(done)
            : "r"(bar), "r"(parity));
        if (!done && it >= limit) return false;
    }
    return true;
}

// The row chunks of one tile that a thread loads: warp instruction j of warp
// w covers rows 8 rg .. 8 rg + 7 (lane % 8) and the 16-byte columns
// 4 cg .. 4 cg + 3 (lane / 8), with (rg, cg) = item j*4 + w of
// 16 row groups x ceil(K/16) column groups.
struct ChunkPos {
    int r, c4;
    bool ok;
};
__device__ __forceinline__ ChunkPos chunk_pos(int j, int wid, int lane, int K)
{
    const int ncg = (K + 15) >> 4;
    const int item = j * 4 + wid;
    const int rg = item / ncg, cg = item - rg * ncg;
    ChunkPos p;
    p.r = rg * 8 + (lane & 7);
    p.c4 = cg * 4 + (lane >> 3);
    p.ok = rg < 16 && p.c4 < (K >> 2);
    return p;
}

// BULK: the tiles of C come through the bulk-copy engine into a ring of
// `stages` shared-memory stages (a tile's rows are contiguous in C: one
// cp.async.bulk per tile, completing on the stage's mbarrier), so that
// several tiles are in flight per CTA without holding them in registers; C
// must be 16-byte aligned.  Otherwise each thread loads its chunks of the
// next tile into registers.
template <bool BULK>
__global__ void __launch_bounds__(kBasisThreads)
k_basis_expand(const float *__restrict__ C, long long M, int K, const float *__restrict__ B, int N,
               float *__restrict__ I, unsigned *__restrict__ err, int aligned, int aligned_b, int test_timeout,
               int stages)
{
    extern __shared__ __align__(1024) unsigned char sm[];
    const int a_bytes = kTileM * K * 4, b_bytes = N * K * 4;
    const int rs = K * 4;                        // a stage row: the tile as it lies in C
    const int nst = BULK ? stages : 0;
    unsigned char *a_hi = sm, *a_lo = sm + a_bytes;
    unsigned char *b_hi = sm + 2 * a_bytes, *b_lo = b_hi + b_bytes;
    unsigned char *raw = b_lo + b_bytes;         // [stages][128][rs] (BULK)
    uint64_t *mbar = reinterpret_cast<uint64_t *>(raw + (size_t)nst * kTileM * rs);   // [2]: one per accumulator
    uint64_t *idle = mbar + 2;   // a barrier nothing arrives at (the time-out test)
    uint64_t *full = mbar + 3;   // [stages]: a stage's copies have landed (BULK)
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(full + nst);
    const int tid = threadIdx.x, wid = tid >> 5, lane = tid & 31;
    const long long tiles = (M + kTileM - 1) / kTileM;
    const int nitems = 16 * ((K + 15) >> 4);   // warp instructions per tile, all warps
    const int per_warp = (nitems + 3) >> 2;

    uint32_t ncols = 32;   // accumulator columns: a power of two >= N, two accumulators
    while (ncols < (uint32_t)N) ncols <<= 1;
    if (wid == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(2 * ncols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(mbar)));
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(mbar + 1)));
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(idle)));
        for (int st = 0; st < nst; st++) asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(full + st)));
        asm volatile("fence.mbarrier_init.release.cluster;");
    }
    // the basis, split into TF32 pairs, once: B[k][n .. n+3] per load (N is
    // a multiple of 16), four loads in flight per thread
    {
        const int n4 = N >> 2;
#pragma unroll 4
        for (int i = tid; i < n4 * K; i += kBasisThreads) {
            const int k = i / n4, n = 4 * (i - k * n4);
            const float *src = B + (size_t)k * N + n;
            float x[4];
            if (aligned_b) {
                const float4 v = __ldg(reinterpret_cast<const float4 *>(src));
                x[0] = v.x; x[1] = v.y; x[2] = v.z; x[3] = v.w;
            } else {
                x[0] = __ldg(src); x[1] = __ldg(src + 1); x[2] = __ldg(src + 2); x[3] = __ldg(src + 3);
            }
#pragma unroll
            for (int q = 0; q < 4; q++) {
                const float hi = tf32_rna(x[q]), lo = tf32_rna(x[q] - hi);
                const int o = kmajor_offset(n + q, k, K);
                *reinterpret_cast<float *>(b_hi + o) = hi;
                *reinterpret_cast<float *>(b_lo + o) = lo;
            }
        }
    }

    // BULK: one thread copies tile t's rows (contiguous in C, 16-byte
    // aligned, a multiple of 32 bytes) into stage st with one bulk copy that
    // completes on the stage's barrier
    auto issue_bulk = [&](long long t, int st) {
        const long long m0 = t * kTileM;
        const int rows = (int)(M - m0 < kTileM ? M - m0 : kTileM);
        const uint32_t fb = smem_u32(full + st);
        const uint32_t bytes = (uint32_t)(rows * K * 4);
        // the split's reads of this stage (generic proxy) before the copy's writes (async proxy)
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(fb), "r"(bytes) : "memory");
        asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                         smem_u32(raw + (size_t)st * kTileM * rs)),
                     "l"(C + m0 * K), "r"(bytes), "r"(fb)
                     : "memory");
    };
    // BULK: stage st, split, into the K-major A buffers (rows past the end of
    // C hold stale words; their accumulator rows are never stored)
    auto split_stage = [&](int st) {
        const unsigned char *src = raw + (size_t)st * kTileM * rs;
#pragma unroll
        for (int j = 0; j < kMaxK / 4; j++) {
            if (j < per_warp) {
                const ChunkPos p = chunk_pos(j, wid, lane, K);
                if (p.ok) {
                    const float4 x = *reinterpret_cast<const float4 *>(src + p.r * rs + 16 * p.c4);
                    float4 h, l;
                    h.x = tf32_rna(x.x); l.x = tf32_rna(x.x - h.x);
                    h.y = tf32_rna(x.y); l.y = tf32_rna(x.y - h.y);
                    h.z = tf32_rna(x.z); l.z = tf32_rna(x.z - h.z);
                    h.w = tf32_rna(x.w); l.w = tf32_rna(x.w - h.w);
                    const int o = kmajor_offset(p.r, 4 * p.c4, K);
                    *reinterpret_cast<float4 *>(a_hi + o) = h;
                    *reinterpret_cast<float4 *>(a_lo + o) = l;
                }
            }
        }
    };

    // this thread's chunks of a tile of C, loaded into registers ahead of use
    float4 ra[BULK ? 1 : kMaxK / 4];
    auto load_tile = [&](long long tile) {
        const long long m0 = tile * kTileM;
#pragma unroll
        for (int j = 0; j < (BULK ? 0 : kMaxK / 4); j++) {
            ra[j] = make_float4(0.f, 0.f, 0.f, 0.f);
            if (j < per_warp) {
                const ChunkPos p = chunk_pos(j, wid, lane, K);
                const long long row = m0 + p.r;
                if (p.ok && row < M) {
                    const float *src = C + row * K + 4 * p.c4;
                    if (aligned) {
                        ra[j] = __ldg(reinterpret_cast<const float4 *>(src));
                    } else {
                        ra[j] = make_float4(__ldg(src), __ldg(src + 1), __ldg(src + 2), __ldg(src + 3));
                    }
                }
            }
        }
    };
    // the registers, split, into the K-major A buffers
    auto store_tile = [&]() {
#pragma unroll
        for (int j = 0; j < (BULK ? 0 : kMaxK / 4); j++) {
            if (j < per_warp) {
                const ChunkPos p = chunk_pos(j, wid, lane, K);
                if (p.ok) {
                    const float4 x = ra[j];
                    float4 h, l;
                    h.x = tf32_rna(x.x); l.x = tf32_rna(x.x - h.x);
                    h.y = tf32_rna(x.y); l.y = tf32_rna(x.y - h.y);
                    h.z = tf32_rna(x.z); l.z = tf32_rna(x.z - h.z);
                    h.w = tf32_rna(x.w); l.w = tf32_rna(x.w - h.w);
                    const int o = kmajor_offset(p.r, 4 * p.c4, K);
                    *reinterpret_cast<float4 *>(a_hi + o) = h;
                    *reinterpret_cast<float4 *>(a_lo + o) = l;
                }
            }
        }
    };
    const uint32_t idesc = idesc_tf32(kTileM, N);
    const uint32_t lbo = 128, sbo = (uint32_t)(K >> 2) * 128;
    auto issue_mma = [&](uint32_t tmem_acc, int b) {
        uint32_t acc = 0;
        for (int pass = 0; pass < 3; pass++) {
            const unsigned char *A = (pass == 2) ? a_lo : a_hi;
            const unsigned char *Bm = (pass == 1) ? b_lo : b_hi;
            for (int kk = 0; kk < K; kk += 8) {
                const uint64_t ad = smem_desc(smem_u32(A + (kk >> 2) * 128), lbo, sbo);
                const uint64_t bd = smem_desc(smem_u32(Bm + (kk >> 2) * 128), lbo, sbo);
                asm volatile(
                    "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                    "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem_acc),
                    "l"(ad), "l"(bd), "r"(idesc), "r"(acc));
                acc = 1;
            }
        }
        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
            smem_u32(mbar + b)));
    };

    long long tile = blockIdx.x;
    if (!BULK && tile < tiles) load_tile(tile);
    // make the barrier initialisation, the basis and the tensor-memory
    // address visible to every thread
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    const uint32_t tmem = *tmem_slot;
    // BULK: the first `stages` tiles of this CTA in flight
    long long issued = -1;   // the last tile index g (in this CTA's order) whose copies were issued
    if (BULK && tid == 0) {
        for (int st = 0; st < nst; st++) {
            const long long t = tile + (long long)st * gridDim.x;
            if (t < tiles) issue_bulk(t, st);
        }
    }
    if (BULK) {
        const long long mine = tile < tiles ? (tiles - 1 - tile) / gridDim.x : -1;   // this CTA's last g
        issued = mine < nst - 1 ? mine : nst - 1;
    }
    uint32_t full_phase = 0u;   // bit st: the next phase of stage st's barrier
    long long consumed = -1;    // the last tile index g whose stage has landed

    // accumulator acc_i (tile ptile) back to HBM: warp w holds lanes
    // 32w .. 32w+31 = rows of the tile; 32 columns per wait
    auto read_back = [&](int acc_i, long long ptile) {
        const long long row = ptile * kTileM + wid * 32 + lane;
        const uint32_t tbase = tmem + ((uint32_t)(wid * 32) << 16) + (uint32_t)acc_i * ncols;
        for (int c = 0; c < N; c += 32) {
            uint32_t v[32];
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, "
                "%12, %13, %14, %15}, [%16];"
                : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
                  "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]),
                  "=r"(v[15])
                : "r"(tbase + (uint32_t)c));
            const bool two = c + 16 < N;
            if (two)
                asm volatile(
                    "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, "
                    "%12, %13, %14, %15}, [%16];"
                    : "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]),
                      "=r"(v[23]), "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]),
                      "=r"(v[30]), "=r"(v[31])
                    : "r"(tbase + (uint32_t)(c + 16)));
            asm volatile("tcgen05.wait::ld.sync.aligned;");
            if (row < M) {
                float *o = I + row * N + c;
                const int nq = two ? 8 : 4;
                if (aligned) {
#pragma unroll
                    for (int q = 0; q < 8; q++)
                        if (q < nq)
                            reinterpret_cast<float4 *>(o)[q] =
                                make_float4(__uint_as_float(v[4 * q]), __uint_as_float(v[4 * q + 1]),
                                            __uint_as_float(v[4 * q + 2]), __uint_as_float(v[4 * q + 3]));
                } else {
#pragma unroll
                    for (int q = 0; q < 32; q++)
                        if (q < 4 * nq) o[q] = __uint_as_float(v[q]);
                }
            }
        }
    };

    bool ok = true;
    uint32_t phase[2] = {0u, 0u};   // the next phase each accumulator's barrier completes
    int pending = -1;               // accumulator whose MMAs are committed and not yet read back
    long long pending_tile = -1;
    int g = 0;
    for (; tile < tiles; g++, tile += gridDim.x) {
        const int b = g & 1;
        const int st = BULK ? g % nst : 0;
        if (BULK) {
            // this tile's stage has landed
            ok = __syncthreads_and(mbar_wait(smem_u32(full + st), (full_phase >> st) & 1u, kSpinLimit)) != 0;
            if (!ok) break;
            full_phase ^= 1u << st;
            consumed = g;
        }
        // the A buffers are free once the previous tile's MMAs are done
        if (pending >= 0) {
            const uint32_t bar = smem_u32(test_timeout ? idle : mbar + pending);
            ok = mbar_wait(bar, phase[pending], test_timeout ? 1024u : kSpinLimit);
            ok = __syncthreads_and(ok) != 0;   // one decision for the block
            if (!ok) break;   // the drain below still waits for the committed MMAs
            asm volatile("tcgen05.fence::after_thread_sync;");
        }
        if (BULK) split_stage(st);
        else store_tile();
        asm volatile("fence.proxy.async.shared::cta;");   // generic-proxy stores -> tensor core
        asm volatile("tcgen05.fence::before_thread_sync;");
        __syncthreads();
        asm volatile("tcgen05.fence::after_thread_sync;");
        if (tid == 0) issue_mma(tmem + (uint32_t)b * ncols, b);
        if (BULK) {
            // the stage is free again (every thread has split it): the tile
            // `stages` ahead goes into it
            const long long nt = tile + (long long)nst * gridDim.x;
            if (nt < tiles) {
                if (tid == 0) issue_bulk(nt, st);
                issued = g + nst;
            }
        } else {
            // next tile's rows into registers while the MMAs run
            const long long next = tile + gridDim.x;
            if (next < tiles) load_tile(next);
        }
        // the previous tile's accumulator back to HBM
        if (pending >= 0) {
            read_back(pending, pending_tile);
            phase[pending] ^= 1u;
        }
        pending = b;
        pending_tile = tile;
    }
    // the last tile: wait, then read it back (or, after a time-out, only let
    // the committed MMAs finish before the tensor memory is freed)
    if (pending >= 0) {
        // the time-out test: a block with a single tile gives up here
        if (test_timeout && ok) ok = __syncthreads_and(mbar_wait(smem_u32(idle), 0u, 1024u)) != 0;
        bool drained = mbar_wait(smem_u32(mbar + pending), phase[pending], kSpinLimit);
        drained = __syncthreads_and(drained) != 0;
        asm volatile("tcgen05.fence::after_thread_sync;");
        if (!ok) {
            if (lane == 0) atomicOr(err, 1u);
            if (!drained && lane == 0) atomicOr(err, 2u);
        } else if (!drained) {
            if (lane == 0) atomicOr(err, 3u);
        } else {
            read_back(pending, pending_tile);
        }
    }
    if (BULK && !ok) {
        // after a time-out: let the copies still in flight land before the
        // block exits (tiles consumed+1 .. issued; a stage holds one copy at
        // a time)
        bool landed = true;
        for (long long gg = consumed + 1; gg <= issued; gg++) {
            const int st = (int)(gg % (nst > 0 ? nst : 1));
            landed = mbar_wait(smem_u32(full + st), (full_phase >> st) & 1u, kSpinLimit) && landed;
            full_phase ^= 1u << st;
        }
        if (!__syncthreads_and(landed) && tid == 0) atomicOr(err, 4u);
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    if (wid == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(2 * ncols));
}

} // namespace

// Shared memory of the register path (the bound xrdt_basis_expand checks);
// the bulk path adds its stages of padded rows and their barriers.
size_t basis_smem(int K, int N) { return 2 * (size_t)kTileM * K * 4 + 2 * (size_t)N * K * 4 + 32; }

namespace {

size_t basis_smem_bulk(int K, int N, int stages)
{
    return basis_smem(K, N) + (size_t)stages * kTileM * K * 4 + 8 * (size_t)stages;
}

template <bool BULK>
cudaError_t launch_basis_variant(const float *C, long long M, int K, const float *B, int N, float *I, unsigned *err,
                                 cudaStream_t s, size_t smem, int stages, int aligned, int aligned_b, int sms,
                                 int smem_sm, int optin)
{
    cudaError_t e = cudaFuncSetAttribute(k_basis_expand<BULK>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
    if (e != cudaSuccess) return e;
    // CTAs per SM: as many as registers and shared memory allow, but no more
    // than the 512 tensor-memory columns hold (two accumulators each, and an
    // allocation that does not fit would wait for another CTA to finish all
    // its tiles); extra shared memory per CTA keeps the block scheduler from
    // placing more
    int ncols = 32;
    while (ncols < N) ncols <<= 1;
    const int tmem_ctas = 512 / (2 * ncols);
    cudaFuncAttributes fa;
    e = cudaFuncGetAttributes(&fa, k_basis_expand<BULK>);
    if (e != cudaSuccess) return e;
    // registers are allocated per warp in units of 256
    const int regs_warp = ((fa.numRegs * 32 + 255) / 256) * 256;
    const int reg_ctas = regs_warp > 0 ? 65536 / (regs_warp * (kBasisThreads / 32)) : 16;
    const size_t per_cta = smem + fa.sharedSizeBytes + 1024;   // 1 KB reserved per block
    const int smem_ctas = (int)((size_t)smem_sm / per_cta);
    int ctas = tmem_ctas;
    if (reg_ctas < ctas) ctas = reg_ctas;
    if (smem_ctas < ctas) ctas = smem_ctas;
    if (ctas > 16) ctas = 16;
    if (ctas < 1) return cudaErrorInvalidConfiguration;
    if (smem_ctas > tmem_ctas && reg_ctas > tmem_ctas) {
        const size_t padded = (size_t)smem_sm / (tmem_ctas + 1) + 1 - fa.sharedSizeBytes - 1024;
        if (padded > smem && padded <= (size_t)optin) smem = padded;
    }
    const long long tiles = (M + kTileM - 1) / kTileM;
    long long grid = (long long)sms * ctas;
    if (grid > tiles) grid = tiles;
    // XRDT_TEST_BASIS_TIMEOUT=1 makes every block's first accumulator wait
    // run out (test of the time-out path: error flag, drain, tensor memory
    // freed)
    const char *tt = getenv("XRDT_TEST_BASIS_TIMEOUT");
    const int test_timeout = (tt && tt[0] == '1') ? 1 : 0;
    k_basis_expand<BULK><<<(unsigned)grid, kBasisThreads, smem, s>>>(C, M, K, B, N, I, err, aligned, aligned_b,
                                                                       test_timeout, stages);
    return cudaGetLastError();
}

} // namespace

cudaError_t launch_basis_expand(const float *C, long long M, int K, const float *B, int N, float *I, unsigned *err,
                                cudaStream_t s, int64_t *launches)
{
    if (M <= 0) return cudaSuccess;
    int dev = 0, sms = 0, smem_sm = 0, optin = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (e != cudaSuccess) return e;
    if (basis_smem(K, N) > (size_t)optin) return cudaErrorInvalidConfiguration;
    const int aligned = (((uintptr_t)C | (uintptr_t)I) & 15) == 0 ? 1 : 0;
    const int aligned_b = ((uintptr_t)B & 15) == 0 ? 1 : 0;
    if (launches) (*launches)++;
    // the bulk-copy ring when C allows it: two or three stages, whichever
    // leaves more CTAs on an SM (the per-tile work is latency-bound, so CTAs
    // count for more than a third stage), three on a tie
    if (((uintptr_t)C & 15) == 0) {
        int best = 0, best_ctas = 0;
        for (int stages = 3; stages >= 2; stages--) {
            const size_t sm_b = basis_smem_bulk(K, N, stages);
            if (sm_b > (size_t)optin) continue;
            const int c = (int)((size_t)smem_sm / (sm_b + 1024));
            if (c > best_ctas) {
                best = stages;
                best_ctas = c;
            }
        }
        if (best)
            return launch_basis_variant<true>(C, M, K, B, N, I, err, s, basis_smem_bulk(K, N, best), best, aligned,
                                              aligned_b, sms, smem_sm, optin);
    }
    return launch_basis_variant<false>(C, M, K, B, N, I, err, s, basis_smem(K, N), 0, aligned, aligned_b, sms,
                                       smem_sm, optin);
}

} // namespace xrdt
