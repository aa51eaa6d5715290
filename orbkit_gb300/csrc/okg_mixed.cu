// Mixed-precision fused density kernel: AO generation on the CUDA cores, the
// C.AO contraction on the 5th-generation tensor cores (tcgen05, BF16 operands,
// FP32 accumulation in TMEM), the density reduction in FP64.
//
// Reference computation: orbkit/core.py:179-304 (slice_rho: AO -> MO ->
// rho = sum occ MO^2, d rho = sum 2 occ dMO MO) with the AO kernel of
// orbkit/c_grid-based.c:9-79.
//
// Precision scheme (all errors against the FP64 oracle are measured by the tests):
//   * exponent argument u = alpha*log2(e) * r^2 in FP64 (r^2 from FP64 coordinates);
//     u is split exactly into a float integer part and fraction with integer bit
//     operations, 2^-f is a degree-7 Taylor polynomial of exp in FP32 (Horner/FMA),
//     2^-k is applied to the float exponent field;
//   * radial sums, polynomials and angular factors in FP32;
//   * each AO value v (FP32) is split v = b0 + b1 + b2 into three BF16 numbers,
//     each MO coefficient (FP64) likewise; six MMAs per (channel, K-step) form
//     b0c0 + b0c1 + b1c0 + b0c2 + b1c1 + b2c0 (the omitted products are below
//     2^-24 relative), accumulated in FP32 in tensor memory.  The tensor core
//     truncates its FP32 accumulation, so every MMA into a large accumulator can
//     lose up to an ulp of it; for the value channel (the one rho is built from)
//     the leading b0c0 products of K-step k go to accumulator k mod 4 and the five
//     small correction products to a fifth, and the five are summed in the
//     epilogue.  Gradient channels use one accumulator each.
//   * rho and grad rho accumulate the per-MO products in FP64.
//
// Tile: 128 grid points (the MMA's M), N = MO block padded to a multiple of 16
// (<= 64 per pass), K = canonical Cartesian AO columns in chunks of 32 (one
// 64-byte swizzle row of BF16).  Persistent CTAs, one per SM, each with
// 128 x NG generation threads (NG threads per grid point), one MMA warp and one
// tile warp.  The tile warp takes tiles from a device counter, screens them and
// assigns their shells to the generation groups, up to two tiles ahead (three
// buffers of tile index, descriptor and screening tables, handed over through
// "screened" and "kfree" mbarriers).  Generation threads and the MMA warp are
// connected by a two-stage ring in shared memory:
//   * generation threads write 4 channels x 3 parts of A (128 x 32 BF16, M-major,
//     SWIZZLE_128B) for a chunk into a free stage and arrive on its "full" barrier;
//   * the MMA warp bulk-copies the chunk's pre-split, pre-swizzled B block into the
//     stage (columns of screened shells then zeroed), waits for "full", issues up to
//     48 MMAs from one thread (descriptors advanced in their 32-bit address word) and
//     commits them to the stage's "empty" barrier, so the tensor core works on one
//     chunk while the next one is generated;
//   * after the last chunk of an MO pass the MMA warp commits to "acc full"; the
//     generation warps read the accumulators (8 x N FP32 columns of TMEM: value
//     4 leading + 1 correction; d/dx, d/dy, d/dz), arrive on "acc empty" and
//     reduce in FP64, each warp owning whole outputs (rho, or one gradient
//     component) of its 32 points.
// Every wait is bounded and raises the status word instead of hanging.
#include <stdio.h>
#include <string.h>

#include <cuda_bf16.h>

#include <vector>

#include "okg_internal.cuh"

namespace okg {
namespace mx {

constexpr int M = 128;
constexpr int KC = OKG_MKC;           // 32 BF16 = 64 bytes
constexpr int ROWB = KC * 2;          // bytes of one operand row
constexpr int RUNITS = ROWB / 16;     // 16-byte units of one operand row
constexpr int A_TILE = M * ROWB;      // bytes of one 128 x 32 BF16 sub-tile
constexpr int A_STAGE = 12 * A_TILE;  // 4 channels x 3 parts
constexpr int NMAX = 64;              // MO columns per pass
constexpr int B_STAGE = 3 * NMAX * ROWB;
constexpr int NSTAGE = 2;
constexpr long long WAIT_LIMIT = 1ll << 24;

__device__ __forceinline__ uint32_t smem_u32(const void* p)
{
    return (uint32_t)__cvta_generic_to_shared(p);
}

// SMEM matrix descriptor of the B operand: K-major, SWIZZLE_64B, SBO = 512 B
// (8-row group stride).
__device__ __forceinline__ uint64_t sdesc(uint32_t addr)
{
    uint64_t d = 0;
    d |= (uint64_t)((addr >> 4) & 0x3FFF);
    d |= (uint64_t)1 << 16;                 // leading byte offset (unused for swizzled K-major)
    d |= (uint64_t)(8 * ROWB >> 4) << 32;   // stride byte offset
    d |= (uint64_t)1 << 46;                 // descriptor version
    d |= (uint64_t)4 << 61;                 // SWIZZLE_64B
    return d;
}

// SMEM matrix descriptor of the A operand: M-major (grid points contiguous),
// SWIZZLE_128B: atoms of 64 points x 8 K (1024 B), the two 64-point halves of the
// tile 1024 B apart (leading byte offset), 8-K groups 2048 B apart (stride byte
// offset).
__device__ __forceinline__ uint64_t adesc_mn(uint32_t addr)
{
    uint64_t d = 0;
    d |= (uint64_t)((addr >> 4) & 0x3FFF);
    d |= (uint64_t)(1024 >> 4) << 16;       // leading byte offset: next 64 points
    d |= (uint64_t)(2048 >> 4) << 32;       // stride byte offset: next 8 K
    d |= (uint64_t)1 << 46;                 // descriptor version
    d |= (uint64_t)2 << 61;                 // SWIZZLE_128B
    return d;
}

// Instruction descriptor: kind::f16, A = B = BF16, D = F32, M-major A, K-major B.
__host__ __device__ constexpr uint32_t idesc_bf16(int M_, int N_)
{
    return (1u << 4) | (1u << 7) | (1u << 10) | (1u << 15) | ((uint32_t)(N_ >> 3) << 17) |
           ((uint32_t)(M_ >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc)
{
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d_tmem),
        "l"(a), "l"(b), "r"(idesc), "r"(acc));
}

// The same MMA with the descriptors as (address word, upper word) pairs: offsets
// inside a stage are added to the address word alone (the start address field,
// shared address >> 4, stays below 2^14 and never carries into the upper bits).
__device__ __forceinline__ void mma_bf16_w(uint32_t d_tmem, uint32_t a_lo, uint32_t a_hi, uint32_t b_lo, uint32_t b_hi,
                                           uint32_t idesc, uint32_t acc)
{
    asm volatile(
        "{\n\t.reg .pred p;\n\t.reg .b64 ad, bd;\n\tmov.b64 ad, {%1, %2};\n\tmov.b64 bd, {%3, %4};\n\t"
        "setp.ne.b32 p, %6, 0;\n\ttcgen05.mma.cta_group::1.kind::f16 [%0], ad, bd, %5, p;\n\t}\n" ::"r"(d_tmem),
        "r"(a_lo), "r"(a_hi), "r"(b_lo), "r"(b_hi), "r"(idesc), "r"(acc));
}

__device__ __forceinline__ void mma_commit(uint32_t bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ bool mbar_try(uint32_t bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}

// Bounded wait: returns false (and raises the status word) if the phase does not
// complete within `limit` polls (WAIT_LIMIT unless the plan sets another).
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, int* status, long long limit)
{
    for (long long it = 0; it < limit; ++it)
        if (mbar_try(bar, parity)) return true;
    atomicExch(status, 1);
    return false;
}

// Wait for the completion of the CTA's own asynchronous work (a bulk copy or
// MMAs) before it leaves: bounded by WAIT_LIMIT whatever the plan's limit, since
// such work always completes; false if even that expires.
__device__ __forceinline__ bool mbar_drain(uint32_t bar, uint32_t parity)
{
    for (long long it = 0; it < WAIT_LIMIT; ++it)
        if (mbar_try(bar, parity)) return true;
    return false;
}

// Whether any thread of the CTA raised the abort flag, the same answer for every
// lane of the calling warp (all 32 lanes must call it): decisions that lead to
// warp-collective instructions (tcgen05.ld, shuffles) stay uniform.
__device__ __forceinline__ bool warp_aborted(const int* flag)
{
    return __any_sync(0xffffffffu, *(const volatile int*)flag != 0);
}

__device__ __forceinline__ void mbar_arrive(uint32_t bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

// One bulk copy global -> shared (16-byte aligned addresses, size a multiple of
// 16) completing on an mbarrier that expects `bytes` transaction bytes.
__device__ __forceinline__ void bulk_load(uint32_t dst, const void* src, uint32_t bytes, uint32_t bar)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
                 "l"(src), "r"(bytes), "r"(bar)
                 : "memory");
}

__device__ __forceinline__ void fence_proxy_async()
{
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void tmem_ld8(uint32_t taddr, uint32_t (&r)[8])
{
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
                 : "r"(taddr));
}

// tcgen05.wait::ld with the destination registers of the preceding loads as
// read-write operands: no use of them can be scheduled before the wait.
__device__ __forceinline__ void tmem_wait_ld5(uint32_t (&r)[5][8])
{
    asm volatile("tcgen05.wait::ld.sync.aligned;"
                 : "+r"(r[0][0]), "+r"(r[0][1]), "+r"(r[0][2]), "+r"(r[0][3]), "+r"(r[0][4]), "+r"(r[0][5]), "+r"(r[0][6]), "+r"(r[0][7]), "+r"(r[1][0]), "+r"(r[1][1]), "+r"(r[1][2]), "+r"(r[1][3]), "+r"(r[1][4]), "+r"(r[1][5]), "+r"(r[1][6]), "+r"(r[1][7]), "+r"(r[2][0]), "+r"(r[2][1]), "+r"(r[2][2]), "+r"(r[2][3]), "+r"(r[2][4]), "+r"(r[2][5]), "+r"(r[2][6]), "+r"(r[2][7]), "+r"(r[3][0]), "+r"(r[3][1]), "+r"(r[3][2]), "+r"(r[3][3]), "+r"(r[3][4]), "+r"(r[3][5]), "+r"(r[3][6]), "+r"(r[3][7]), "+r"(r[4][0]), "+r"(r[4][1]), "+r"(r[4][2]), "+r"(r[4][3]), "+r"(r[4][4]), "+r"(r[4][5]), "+r"(r[4][6]), "+r"(r[4][7]));
}

// tcgen05.wait::ld with the destination registers of the preceding loads as
// read-write operands: no use of them can be scheduled before the wait.
__device__ __forceinline__ void tmem_wait_ld1(uint32_t (&r)[1][8])
{
    asm volatile("tcgen05.wait::ld.sync.aligned;"
                 : "+r"(r[0][0]), "+r"(r[0][1]), "+r"(r[0][2]), "+r"(r[0][3]), "+r"(r[0][4]), "+r"(r[0][5]), "+r"(r[0][6]), "+r"(r[0][7]));
}

__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// Exact conversion of a double to float by truncating the mantissa (integer ops
// only; values below 2^-126 in magnitude become 0).
__device__ __forceinline__ float dbl_to_flt_trunc(double d)
{
    const int hi = __double2hiint(d);
    const unsigned lo = (unsigned)__double2loint(d);
    const int e = (hi >> 20) & 0x7FF;
    if (e <= 896) return 0.0f;
    const unsigned bits = ((unsigned)hi & 0x80000000u) | ((unsigned)(e - 896) << 23) |
                          (((unsigned)hi & 0xFFFFFu) << 3) | (lo >> 29);
    return __uint_as_float(bits);
}

// e^(-u ln 2) = 2^-u for an FP64 argument u >= 0 (u = alpha log2(e) r^2).
// u = uh + r exactly with uh the float truncation of u (its top 24 significant bits)
// and r the remaining 29 mantissa bits, both taken from the bit pattern with integer
// operations: r = (low 29 bits) 2^(e - 1075), converted toward zero to 24 bits (the
// FP64 pipe is not used; below u = 2^-74 r is dropped).  k = rint(uh),
// f = (uh - k) + r in FP32 (uh - k is exact), |f| <= 0.5 + 2^-23.  2^-f by the
// degree-7 Taylor series of exp(y), y = -f ln 2 (|y| < 0.35, truncation error
// < 6e-9 relative), scaled by 2^-k through the exponent field.
__device__ __forceinline__ float exp2_neg(double u)
{
    if (__double2hiint(u) >= 0x40690000) return 0.0f;  // u >= 200: 2^-u underflows in float
    const int hi = __double2hiint(u);
    const unsigned lo = (unsigned)__double2loint(u);
    const double uh_d = __hiloint2double(hi, (int)(lo & 0xE0000000u));
    const int e = (hi >> 20) & 0x7FF;
    const float uh = dbl_to_flt_trunc(uh_d);
    const float rf = e >= 949 ? __uint2float_rz(lo & 0x1FFFFFFFu) * __int_as_float((e - 948) << 23) : 0.0f;
    const float k = rintf(uh);
    const float f = (uh - k) + rf;
    const float y = -f * 0.693147180559945309f;
    float p = 1.0f / 5040.0f;
    p = fmaf(p, y, 1.0f / 720.0f);
    p = fmaf(p, y, 1.0f / 120.0f);
    p = fmaf(p, y, 1.0f / 24.0f);
    p = fmaf(p, y, 1.0f / 6.0f);
    p = fmaf(p, y, 0.5f);
    p = fmaf(p, y, 1.0f);
    p = fmaf(p, y, 1.0f);
    const int ki = (int)k;
    const int ebits = (int)((__float_as_uint(p) >> 23) & 0xFF) - ki;
    if (ebits <= 0) return 0.0f;
    return __uint_as_float(__float_as_uint(p) - ((unsigned)ki << 23));
}

// Split an FP32 value into three BF16 values with v = b0 + b1 + b2 to 2^-24.
__device__ __forceinline__ void split3(float v, __nv_bfloat16& b0, __nv_bfloat16& b1, __nv_bfloat16& b2)
{
    b0 = __float2bfloat16_rn(v);
    const float r1 = v - __bfloat162float(b0);
    b1 = __float2bfloat16_rn(r1);
    const float r2 = r1 - __bfloat162float(b1);
    b2 = __float2bfloat16_rn(r2);
}

// byte offset of element (row m, column k) in a K-major BF16 tile with 32-element
// rows and SWIZZLE_64B (the B operand): 8-row groups of 512 B, the 16-byte unit
// index XORed with address bits 7..8, i.e. (m >> 1) & 3
__host__ __device__ __forceinline__ uint32_t sw64_off(int m, int k)
{
    return (uint32_t)((m >> 3) * 512 + (m & 7) * 64 + ((((k >> 3) ^ (m >> 1)) & 3) << 4) + ((k & 7) << 1));
}

// byte offset of element (point m, column k) of the 128 x 32 M-major SWIZZLE_128B A
// tile: 128-byte rows of 64 consecutive points for one column, the 16-byte unit
// index XORed with the row's position in its 8-row atom (k % 8)
__device__ __forceinline__ uint32_t amn_off(int m, int k)
{
    return (uint32_t)((m >> 6) * 1024 + (k >> 3) * 2048 + (k & 7) * 128 + ((((m >> 3) ^ k) & 7) << 4) + ((m & 7) << 1));
}

// One molecule as seen by a tile: its basis tables, grid, coefficient tiles and outputs.
struct alignas(16) MolDesc {
    BasisDev B;
    Grid g;
    const uint4* bpack;  // [npass][nmchunk][3][npad x 64 B], pre-swizzled
    const double* occ;   // [npass * npad] occupations, then [npass * npad] 2 x occupations (zero padded)
    const float2* occf;  // the same 2 x npass x npad values as double-float (hi, lo) pairs
    double* rho;
    double* grad;        // 3 x ld
    long long ld;
    long long tile0;     // first tile of this molecule in the batch's tile numbering
    long long ntiles;
    int npass, npad;
    int nmo;             // MO columns beyond nmo (last pass) are zero padding
    int want_grad;
    int brick;           // regular grid covered by 4 x 4 x 8 bricks (else runs of 128 flattened points)
    int nby, nbz;        // bricks along y and z
    // cusp points (null near: none): near[p] = the atom within whose cusp radius point p
    // lies, or -1; there the atom's primitives with alpha > alpha_c are left out of the
    // tensor-core operand and their part of every MO (C_eff in FP64, ceff) is added in
    // FP64 in the epilogue
    const short* near;
    const double* ceff;  // C_eff transposed (ncart x nmo: the MOs of a column contiguous), FP64
    double alpha_c;
    double cusp_pad;
};

// Single-molecule launch.
struct Params {
    MolDesc D;
    int* status;                  // device status word: 1 = timeout
    unsigned long long* counter;  // tile counter, zero at launch (tiles are handed out dynamically)
    long long wait_limit;         // polls per bounded wait
};

// Screening: a primitive is skipped for a tile when alpha log2(e) d^2 > SCREEN_LOG2,
// d = distance from its atom to the tile's bounding box, i.e. its exponential is
// below 2^-64 (5e-20) at every point of the tile.
constexpr float SCREEN_LOG2 = 64.0f;

// Shared-memory pieces of the CTA.  Two tile buffers (tile index, column masks,
// batch descriptor) let the generation threads screen the next tile while the
// MMA warp still works through the previous one.
struct CtaState {
    unsigned char* A_s;          // NSTAGE x A_STAGE
    unsigned char* B_s;          // NSTAGE x B_STAGE
    uint32_t bar_full;           // NSTAGE mbarriers, 8 B apart: stage written by every generation thread
    uint32_t bar_empty;          // NSTAGE mbarriers: the stage's MMAs are complete (tcgen05.commit)
    uint32_t bar_bload;          // NSTAGE mbarriers: the stage's B block has landed (bulk copy)
    uint32_t bar_acc_full;       // accumulators of a job (tile, MO pass) complete (tcgen05.commit)
    uint32_t bar_acc_empty;      // every generation thread has read the accumulators
    uint32_t bar_screened;       // NBUF mbarriers (tile buffers): tile index and screening tables written
    uint32_t bar_kfree;          // NBUF mbarriers: generation threads and MMA warp are done with the buffer's tile
    uint32_t bar_drain;          // the MMA warp's last commit: every MMA it issued is complete
    long long wait_limit;        // polls per bounded wait
    uint32_t tmem;
    int* abort_flag;
    unsigned char* nkeep;        // NBUF x MAX_SHELLS: per shell, kept primitives | owning generation group << 5
    unsigned* kmask;             // NBUF x MAX_CHUNKS: per chunk, columns whose shell is kept for the buffer's tile
    long long* tile_slot;        // NBUF: tile of the buffer (local to its molecule); -1: no more tiles
    int* cusp_atoms;             // NBUF x (1 + NCA): count, then the atoms whose cusp region holds a point of the tile
    MolDesc* mol;                // NBUF: molecule of the buffer's tile (one copy for the single-molecule kernel)
};

// Per-tile screening tables live in shared memory: at most MAX_SHELLS shells and
// MAX_CHUNKS chunks per molecule on the mixed path.
constexpr int MAX_SHELLS = 2048;
// FP64 cusp region: at most NCA atoms whose cusp region holds a point of one tile (more
// raise status bit 2, reported as OKG_ERR_UNSUPPORTED; the first NCA are treated)
constexpr int NCA = 8;
constexpr int MAX_CHUNKS = 192;
// Tile buffers (index, descriptor, screening tables) between the tile warp and the
// generation threads / MMA warp: the tile warp screens up to NBUF - 1 tiles ahead.
constexpr int NBUF = 3;
__device__ __forceinline__ int tbuf(uint32_t ord) { return (int)(ord % NBUF); }
__device__ __forceinline__ uint32_t tphase(uint32_t ord) { return (ord / NBUF) & 1u; }
// A shell's byte of the screening table: kept primitives (low 5 bits, so at most
// MAX_PRIM per shell on the mixed path) and the generation group that evaluates
// the shell for this tile (high 3 bits, at most 8 groups).
constexpr int MAX_PRIM = 31;
constexpr int KEEP_BITS = 5;

// FP64 <-> FP32 without the FP64 pipe: rounding double -> float and exact
// float -> double through integer operations on the IEEE bit patterns.
__device__ __forceinline__ float dbl_to_flt_rn(double d)
{
    unsigned long long u = (unsigned long long)__double_as_longlong(d);
    const unsigned long long mag = u & 0x7FFFFFFFFFFFFFFFull;
    if (mag < 0x3810000000000000ull) return 0.0f;  // |d| < 2^-126
    u += 0x10000000ull;                           // round to nearest at the float's last bit
    const unsigned hi = (unsigned)(u >> 32), lo = (unsigned)u;
    const unsigned e = (hi >> 20) & 0x7FF;
    return __uint_as_float((hi & 0x80000000u) | ((e - 896u) << 23) | ((hi & 0xFFFFFu) << 3) | (lo >> 29));
}

__device__ __forceinline__ double flt_to_dbl(float f)
{
    const unsigned u = __float_as_uint(f);
    const unsigned e = (u >> 23) & 0xFF;
    if (e == 0) return 0.0;  // zero (denormals flushed)
    return __hiloint2double((int)((u & 0x80000000u) | ((e + 896u) << 20) | ((u >> 3) & 0xFFFFFu)), (int)(u << 29));
}

// Double-float (hi + lo, FP32) accumulation: two-sum of the high parts, low parts
// collected separately (Dekker / Knuth); products exact through FMA.
struct DF {
    float hi = 0.f, lo = 0.f;
    __device__ __forceinline__ void add(float2 t)
    {
        const float s = hi + t.x;
        const float bb = s - hi;
        const float err = (hi - (s - bb)) + (t.x - bb);
        hi = s;
        lo += err + t.y;
    }
};

// (o.x + o.y) * (a * b) as a double-float (a * b exact: p + e with e = fma(a, b, -p))
__device__ __forceinline__ float2 df_mul(float2 o, float a, float b)
{
    const float p = a * b;
    const float e = fmaf(a, b, -p);
    const float q = o.x * p;
    const float r = fmaf(o.x, p, -q) + (o.x * e + o.y * p);
    return make_float2(q, r);
}

// A Shell (12 ints, 16-byte aligned in the basis block) as three 16-byte loads.
__device__ __forceinline__ Shell load_shell(const Shell* p)
{
    const int4* q = reinterpret_cast<const int4*>(p);
    const int4 a = __ldg(q), b = __ldg(q + 1), c = __ldg(q + 2);
    Shell s;
    s.atom = a.x; s.L = a.y; s.nprim = a.z; s.prim0 = a.w;
    s.cart0 = b.x; s.ncart = b.y; s.comp0 = b.z; s.out0 = b.w;
    s.nout = c.x; s.sph0 = c.y; s.mcol = c.z; s.mchunk = c.w;
    return s;
}

// Brick coordinates of a tile (32-bit division unless the grid is beyond 2^31 tiles).
__device__ __forceinline__ void brick_of(const MolDesc& D, long long tile, int& bi, int& bj, int& bk)
{
    const long long nbyz = (long long)D.nby * D.nbz;
    int rem;
    if (tile < 0x7FFFFFFFll && nbyz < 0x7FFFFFFFll) {
        bi = (int)tile / (int)nbyz;
        rem = (int)tile - bi * (int)nbyz;
    } else {
        bi = (int)(tile / nbyz);
        rem = (int)(tile - (long long)bi * nbyz);
    }
    bj = rem / D.nbz;
    bk = rem - bj * D.nbz;
}

// The fields of a shell record that chunk generation reads (two of its three
// 16-byte units).
struct GenShell {
    int atom, L, prim0, mcol;
};

__device__ __forceinline__ GenShell load_gen_shell(const Shell* p)
{
    const int4* q = reinterpret_cast<const int4*>(p);
    const int4 a = __ldg(q), c = __ldg(q + 2);
    return GenShell{a.x, a.y, a.w, c.z};
}

// Point of row r of a tile.
__device__ __forceinline__ bool tile_point(const MolDesc& D, long long tile, int r, long long& p)
{
    if (D.brick) {
        int bi, bj, bk;
        brick_of(D, tile, bi, bj, bk);
        const int i = bi * 4 + (r >> 5), j = bj * 4 + ((r >> 3) & 3), k = bk * 8 + (r & 7);
        if (i >= D.g.nx || j >= D.g.ny || k >= D.g.nz) {
            p = 0;
            return false;
        }
        p = ((long long)i * D.g.ny + j) * D.g.nz + k;
        return true;
    }
    p = tile * M + r;
    if (p >= D.g.npts) {
        p = D.g.npts - 1;
        return false;
    }
    return true;
}

// The same with the point's coordinates; a brick reads its axis values directly (a
// row outside the grid gets the nearest grid point's coordinates and p = 0).
__device__ __forceinline__ bool tile_point_xyz(const MolDesc& D, long long tile, int r, long long& p, double& x,
                                               double& y, double& z)
{
    if (D.brick) {
        int bi, bj, bk;
        brick_of(D, tile, bi, bj, bk);
        const int i = bi * 4 + (r >> 5), j = bj * 4 + ((r >> 3) & 3), k = bk * 8 + (r & 7);
        const bool valid = i < D.g.nx && j < D.g.ny && k < D.g.nz;
        x = __ldg(D.g.x + (i < D.g.nx ? i : D.g.nx - 1));
        y = __ldg(D.g.y + (j < D.g.ny ? j : D.g.ny - 1));
        z = __ldg(D.g.z + (k < D.g.nz ? k : D.g.nz - 1));
        p = valid ? ((long long)i * D.g.ny + j) * D.g.nz + k : 0;
        return valid;
    }
    const bool valid = tile_point(D, tile, r, p);
    grid_point(D.g, p, x, y, z);
    return valid;
}

// K-steps (16 columns each) of a kept chunk that hold a kept column: the MMAs of a
// K-step whose columns are all screened are not issued.
__device__ __forceinline__ int ksteps_of(unsigned km)
{
    return ((km & 0xFFFFu) != 0u) + ((km >> 16) != 0u);
}

// Next chunk after c (in chunk order) with a kept column, or -1.
__device__ __forceinline__ int next_kept(const unsigned* km, int nmchunk, int c)
{
    for (++c; c < nmchunk; ++c)
        if (km[c] != 0u) return c;
    return -1;
}

// Where the tiles come from: a device counter over one molecule's tiles, or grabs
// of consecutive tiles of a batch (molecule found by binary search over tile0).
struct TileFeed {
    unsigned long long* counter;  // zero at launch
    long long ntiles;             // tiles of the molecule, or of the whole batch
    const MolDesc* descs;         // batch: nmol descriptors, ascending tile0
    int nmol, grab;
};

// Grid points of a generation thread: P consecutive rows of the tile.
template <int P>
struct GenPts {
    double x[P], y[P], z[P];
};

// The epilogue point of a generation thread (its TMEM lane): coordinates, and the
// cusp atoms of its tile (ncusp of them; the list is copied out of the tile buffer,
// which the tile warp may reuse before the epilogue runs).
struct EpiPt {
    double x, y, z;
    int ncusp;
    int atoms[NCA];
};

// Tile warp (the last warp of the CTA): takes tiles from the feed into buffer
// ord % NBUF once the generation threads and the MMA warp have released that
// buffer's previous tile, computes the tile's bounding box, screens every shell
// against it (primitives kept per shell, kept columns per chunk) and assigns the
// kept shells to generation groups, then arrives on the buffer's "screened"
// barrier.  It runs up to NBUF - 1 tiles ahead of the generation threads, so none
// of this is on their path.  A buffer with tile -1 ends the CTA.
template <int NG, bool BATCH, bool CUSP>
__device__ __forceinline__ void tile_role(const TileFeed& F, const CtaState& S, int* status)
{
    static_assert(NG >= 1 && NG <= (256 >> KEEP_BITS), "generation group index must fit the screening byte");
    const int lane = threadIdx.x & 31;
    long long gnext = 0, gend = 0, gpend = -1;
    for (uint32_t ord = 0;; ++ord) {
        const int b = tbuf(ord);
        if (ord >= NBUF && !mbar_wait(S.bar_kfree + 8 * b, tphase(ord - NBUF), status, S.wait_limit)) *S.abort_flag = 1;
        long long t = -1;
        int mol = 0;
        // the counter increment for the following tile (or range) is issued one
        // fetch ahead (gpend), so its round trip overlaps a tile
        if (lane == 0 && !*S.abort_flag) {
            if (!BATCH) {
                t = gpend >= 0 ? gpend : (long long)atomicAdd(F.counter, 1ull);
                gpend = (long long)atomicAdd(F.counter, 1ull);
                if (t >= F.ntiles) t = -1;
            } else {
                if (gnext >= gend) {
                    gnext = gpend >= 0 ? gpend : (long long)atomicAdd(F.counter, (unsigned long long)F.grab);
                    gpend = -1;
                    gend = gnext + F.grab < F.ntiles ? gnext + F.grab : F.ntiles;
                }
                if (gnext < gend) {
                    t = gnext++;
                    if (gnext == gend && gend < F.ntiles)
                        gpend = (long long)atomicAdd(F.counter, (unsigned long long)F.grab);
                    int lo = 0, hi = F.nmol - 1;
                    while (lo < hi) {
                        const int mid = (lo + hi + 1) >> 1;
                        if (F.descs[mid].tile0 <= t) lo = mid; else hi = mid - 1;
                    }
                    mol = lo;
                }
            }
        }
        t = __shfl_sync(0xffffffffu, t, 0);
        if (BATCH && t >= 0) {
            mol = __shfl_sync(0xffffffffu, mol, 0);
            constexpr int U = (int)(sizeof(MolDesc) / 16);
            const uint4* src = (const uint4*)(F.descs + mol);
            uint4* dst = (uint4*)(S.mol + b);
            for (int i = lane; i < U; i += 32) dst[i] = src[i];
            t -= F.descs[mol].tile0;
        }
        if (lane == 0) S.tile_slot[b] = t;
        __syncwarp();
        if (t < 0) {
            mbar_arrive(S.bar_screened + 8 * b);
            return;
        }
        const MolDesc& D = S.mol[BATCH ? b : 0];
        const BasisDev& B = D.B;
        // bounding box of the tile's valid points
        float v[6] = {3.0e38f, 3.0e38f, 3.0e38f, -3.0e38f, -3.0e38f, -3.0e38f};
        if (D.brick) {
            // a brick spans 4 x, 4 y and 8 z axis values (fewer at the grid's far
            // faces): lanes 0-3, 4-7 and 8-15 take one each
            const long long nbyz = (long long)D.nby * D.nbz;
            const int bi = (int)(t / nbyz);
            const int rem = (int)(t - (long long)bi * nbyz);
            const int bj = rem / D.nbz, bk = rem - bj * D.nbz;
            int axis = -1, idx = 0;
            if (lane < 4) {
                axis = 0;
                idx = bi * 4 + lane;
            } else if (lane < 8) {
                axis = 1;
                idx = bj * 4 + lane - 4;
            } else if (lane < 16) {
                axis = 2;
                idx = bk * 8 + lane - 8;
            }
            const int n_ax = axis == 0 ? D.g.nx : axis == 1 ? D.g.ny : D.g.nz;
            if (axis >= 0 && idx < n_ax) {
                const double* ax = axis == 0 ? D.g.x : axis == 1 ? D.g.y : D.g.z;
                const float c = dbl_to_flt_rn(__ldg(ax + idx));
#pragma unroll
                for (int a = 0; a < 3; ++a)
                    if (a == axis) {
                        v[a] = c;
                        v[3 + a] = c;
                    }
            }
        } else {
            // runs of 128 points: four rows per lane
#pragma unroll
            for (int i = 0; i < M / 32; ++i) {
                long long pg;
                if (tile_point(D, t, lane + 32 * i, pg)) {
                    double x, y, z;
                    grid_point(D.g, pg, x, y, z);
                    const float fx = dbl_to_flt_rn(x), fy = dbl_to_flt_rn(y), fz = dbl_to_flt_rn(z);
                    v[0] = fminf(v[0], fx);
                    v[1] = fminf(v[1], fy);
                    v[2] = fminf(v[2], fz);
                    v[3] = fmaxf(v[3], fx);
                    v[4] = fmaxf(v[4], fy);
                    v[5] = fmaxf(v[5], fz);
                }
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
            for (int c = 0; c < 3; ++c) v[c] = fminf(v[c], __shfl_xor_sync(0xffffffffu, v[c], o));
#pragma unroll
            for (int c = 3; c < 6; ++c) v[c] = fmaxf(v[c], __shfl_xor_sync(0xffffffffu, v[c], o));
        }
        unsigned* km = S.kmask + b * MAX_CHUNKS;
        unsigned char* nkeep = S.nkeep + b * MAX_SHELLS;
        for (int c = lane; c < B.nmchunk; c += 32) km[c] = 0u;
        // the atoms whose cusp region holds a point of the tile (the caller's per-point
        // table), at most NCA; their steep primitives leave the tile's BF16 operand
        int* ca = S.cusp_atoms + b * (1 + NCA);
        int nca = 0;
        int cat[NCA];
        if (CUSP && D.near) {
            int mine[M / 32];
#pragma unroll
            for (int i = 0; i < M / 32; ++i) {
                long long pg;
                mine[i] = tile_point(D, t, lane + 32 * i, pg) ? (int)__ldg(D.near + pg) : -1;
                if (mine[i] >= B.natom) mine[i] = -1;
            }
            for (;;) {
                int cand = -1;
#pragma unroll
                for (int i = 0; i < M / 32; ++i) cand = mine[i] >= 0 ? mine[i] : cand;
                const unsigned any = __ballot_sync(0xffffffffu, cand >= 0);
                if (!any) break;
                const int a = __shfl_sync(0xffffffffu, cand, __ffs(any) - 1);
                if (nca == NCA) {
                    if (lane == 0) atomicOr(status, 2);
                    break;
                }
                cat[nca++] = a;
#pragma unroll
                for (int i = 0; i < M / 32; ++i) mine[i] = mine[i] == a ? -1 : mine[i];
            }
        }
        if (lane == 0) {
            ca[0] = nca;
            for (int i = 0; i < nca; ++i) ca[1 + i] = cat[i];
        }
        const double a2c = D.alpha_c * 1.4426950408889634;
        __syncwarp();
        // a primitive is kept while alpha log2(e) d^2 <= SCREEN_LOG2 (primitives sorted by alpha per shell)
        for (int si = lane; si < B.nshell; si += 32) {
            const Shell sh = load_shell(B.mshells + si);
            const float ax = (float)B.atoms[4 * sh.atom], ay = (float)B.atoms[4 * sh.atom + 1],
                        az = (float)B.atoms[4 * sh.atom + 2];
            const float dx = fmaxf(0.f, fmaxf(v[0] - ax, ax - v[3]));
            const float dy = fmaxf(0.f, fmaxf(v[1] - ay, ay - v[4]));
            const float dz = fmaxf(0.f, fmaxf(v[2] - az, az - v[5]));
            const float d2 = dx * dx + dy * dy + dz * dz;
            // (a count with independent loads: the kept primitives are a prefix)
            int nk = 0;
            for (int k = 0; k < sh.nprim; ++k) nk += (float)B.prim_mx[sh.prim0 + k].a2 * d2 <= SCREEN_LOG2;
            if (CUSP) {
                // a cusp atom of the tile keeps only its smooth primitives (alpha <= alpha_c, a
                // prefix): the epilogue adds the steep ones in FP64 at every point of the tile
                bool cusp_atom = false;
                for (int i = 0; i < nca; ++i) cusp_atom = cusp_atom || cat[i] == sh.atom;
                if (cusp_atom) {
                    int m = 0;
                    while (m < nk && B.prim_mx[sh.prim0 + m].a2 <= a2c) ++m;
                    nk = m;
                }
            }
            nkeep[si] = (unsigned char)nk;
            if (nk > 0) atomicOr(km + sh.mchunk, ((1u << ncanon(sh.L)) - 1u) << sh.mcol);
        }
        __syncwarp();
        // generation groups: per kept chunk (at most 32 shells, one per lane), the kept
        // shells sorted by estimated work (kept primitives and components, bitonic sort
        // across the warp) are dealt to the groups in snake order (0 1 .. NG-1 NG-1 .. 0
        // 0 ..), so every group finishes the chunk at about the same time -- the stage's
        // "full" barrier waits for all of them.  A group recomputes an atom's coordinates
        // when its previous shell belonged to another atom.
        const int wcomp = D.want_grad ? 16 : 5;
        for (int c = 0; c < B.nmchunk; ++c) {
            if (km[c] == 0u) continue;
            const int4 ck = B.mchunks[c];
            const int si = ck.x + lane;
            unsigned key = 0u;  // work << 8 | shell offset; 0: no kept shell
            if (si < ck.y) {
                const int nk = nkeep[si];
                if (nk > 0) key = (unsigned)(3 * nk + wcomp * ncanon(B.mshells[si].L)) << 8 | (unsigned)lane;
            }
#pragma unroll
            for (int k = 2; k <= 32; k <<= 1) {
#pragma unroll
                for (int j = k >> 1; j > 0; j >>= 1) {
                    const unsigned other = __shfl_xor_sync(0xffffffffu, key, j);
                    const bool take_max = ((lane & j) == 0) == ((lane & k) == 0);
                    key = take_max ? max(key, other) : min(key, other);
                }
            }
            if (key != 0u) {
                const int turn = lane / NG, r = lane - turn * NG;
                const int g = (turn & 1) ? NG - 1 - r : r;
                const int sk = ck.x + (int)(key & 0xFFu);
                nkeep[sk] = (unsigned char)(nkeep[sk] | (g << KEEP_BITS));
            }
        }
        __syncwarp();
        mbar_arrive(S.bar_screened + 8 * b);
    }
}

// Generation threads: wait until buffer ord % 2 holds a screened tile; this
// thread's store point (TMEM lane 32 (warp % 4) + lane of the epilogue) and its
// generation points (rows P (tid % (128 / P)) + i).  Returns the tile (local to its
// molecule) or -1 when there are no more.
template <int P, bool BATCH, bool CUSP>
__device__ __forceinline__ long long gen_open_tile(const CtaState& S, uint32_t ord, long long& p, bool& valid,
                                                   GenPts<P>& gp, EpiPt& ep, int* status)
{
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int b = tbuf(ord);
    if (warp_aborted(S.abort_flag)) return -1;
    if (!__all_sync(0xffffffffu, mbar_wait(S.bar_screened + 8 * b, tphase(ord), status, S.wait_limit))) {
        *S.abort_flag = 1;
        return -1;
    }
    const long long tile = S.tile_slot[b];
    if (tile < 0) return -1;
    const MolDesc& D = S.mol[BATCH ? b : 0];
    // the epilogue row 32 (warp % 4) + lane is the generation row when P = 1
    double ex, ey, ez;
    valid = tile_point_xyz(D, tile, 32 * (warp & 3) + lane, p, ex, ey, ez);
    ep.ncusp = 0;
    if constexpr (CUSP) {
        const int* ca = S.cusp_atoms + b * (1 + NCA);
        ep.ncusp = valid ? ca[0] : 0;
        for (int i = 0; i < ep.ncusp; ++i) ep.atoms[i] = ca[1 + i];
        ep.x = ex;
        ep.y = ey;
        ep.z = ez;
    }
    if constexpr (P == 1) {
        gp.x[0] = ex;
        gp.y[0] = ey;
        gp.z[0] = ez;
    } else {
#pragma unroll
        for (int i = 0; i < P; ++i) {
            long long pg;
            tile_point_xyz(D, tile, P * (tid % (128 / P)) + i, pg, gp.x[i], gp.y[i], gp.z[i]);
        }
    }
    return tile;
}

// The generation group evaluating a shell keeps the r^2 and coordinates of the
// shell's atom for the following shells of the same atom.
struct AtomRunBase {
    int last_atom = -1;
};
template <int P>
struct AtomRun : AtomRunBase {
    double rr[P];
    float X[P], Y[P], Z[P];
};

// All canonical components of an L shell at two points, for the channels in
// chmask: sink(channel, canonical index, value at point 0, value at point 1).
template <int L, typename Sink2>
__device__ __forceinline__ void shell_eval2(const float (&X)[2], const float (&Y)[2], const float (&Z)[2],
                                            const Radial<float> (&r)[2], unsigned chmask, Sink2&& sink)
{
    float px[2][L + 3], py[2][L + 3], pz[2][L + 3];
#pragma unroll
    for (int i = 0; i < 2; ++i) {
        px[i][0] = py[i][0] = pz[i][0] = 1.f;
#pragma unroll
        for (int e = 1; e < L + 3; ++e) {
            px[i][e] = px[i][e - 1] * X[i];
            py[i][e] = py[i][e - 1] * Y[i];
            pz[i][e] = pz[i][e - 1] * Z[i];
        }
    }
#pragma unroll
    for (int ch = 0; ch < 4; ++ch) {
        if (!(chmask & (1u << ch))) continue;
        [&]<int... J>(std::integer_sequence<int, J...>) {
            (sink(ch, J,
                  channel_poly<canon_l(L, J, 0), canon_l(L, J, 1), canon_l(L, J, 2), float>(ch, px[0], py[0], pz[0],
                                                                                           r[0], false),
                  channel_poly<canon_l(L, J, 0), canon_l(L, J, 1), canon_l(L, J, 2), float>(ch, px[1], py[1], pz[1],
                                                                                           r[1], false)),
             ...);
        }(std::make_integer_sequence<int, ncanon(L)>{});
    }
}

template <typename Sink2>
__device__ __forceinline__ void shell_eval2_L(int L, const float (&X)[2], const float (&Y)[2], const float (&Z)[2],
                                              const Radial<float> (&r)[2], unsigned chmask, Sink2&& sink)
{
    switch (L) {
    case 0: shell_eval2<0>(X, Y, Z, r, chmask, sink); break;
    case 1: shell_eval2<1>(X, Y, Z, r, chmask, sink); break;
    case 2: shell_eval2<2>(X, Y, Z, r, chmask, sink); break;
    case 3: shell_eval2<3>(X, Y, Z, r, chmask, sink); break;
    default: shell_eval2<4>(X, Y, Z, r, chmask, sink); break;
    }
}

// Generation threads: the AO values (4 or 1 channels x 3 BF16 parts) of one kept
// chunk for this thread's P points and atoms, into the next
// stage of the ring.  With P = 2 the two points are adjacent in the M-major tile:
// each part of a value pair is one packed conversion and one 4-byte store.
template <int NTG, int P>
__device__ __forceinline__ void gen_chunk(const BasisDev& B, const unsigned char* nkeep, int c, const CtaState& S,
                                          uint32_t& seq, AtomRun<P>& ar, unsigned chmask, const GenPts<P>& gp,
                                          int* status)
{
    const int tid = threadIdx.x;
    const int r0 = P * (tid % (128 / P));  // first point row of this thread
    const int grp = tid / (128 / P);
    const uint32_t s = seq & 1u, u = seq >> 1;
    unsigned char* A_s = S.A_s + s * A_STAGE;
    if (u > 0 && !mbar_wait(S.bar_empty + 8 * s, (u - 1) & 1u, status, S.wait_limit)) *S.abort_flag = 1;
    const int4 ck = B.mchunks[c];
    // this group's kept shells of the chunk: the screening bytes are scanned, and the
    // record of the next own shell is loaded one own shell ahead
    auto next_own = [&](int t) {
        for (; t < ck.y; ++t) {
            const int kb = nkeep[t];
            if ((kb & MAX_PRIM) != 0 && (kb >> KEEP_BITS) == grp) break;
        }
        return t;
    };
    int si = next_own(ck.x);
    GenShell nx{0, 0, 0, 0};
    if (si < ck.y) nx = load_gen_shell(B.mshells + si);
    while (si < ck.y) {
        const GenShell sh = nx;
        const int nk = nkeep[si] & MAX_PRIM;
        const int sn = next_own(si + 1);
        if (sn < ck.y) nx = load_gen_shell(B.mshells + sn);
        if (sh.atom != ar.last_atom) {
            ar.last_atom = sh.atom;
            const double ax = B.atoms[4 * sh.atom], ay = B.atoms[4 * sh.atom + 1], az = B.atoms[4 * sh.atom + 2];
#pragma unroll
            for (int i = 0; i < P; ++i) {
                const double X = gp.x[i] - ax, Y = gp.y[i] - ay, Z = gp.z[i] - az;
                ar.rr[i] = X * X + Y * Y + Z * Z;
                ar.X[i] = dbl_to_flt_rn(X);
                ar.Y[i] = dbl_to_flt_rn(Y);
                ar.Z[i] = dbl_to_flt_rn(Z);
            }
        }
        if constexpr (P == 1) {
            // primitives two at a time (two independent exponentials in flight)
            float R0 = 0.f, R1 = 0.f;
            for (int k = 0; k < nk; k += 2) {
                const PrimMx pa = B.prim_mx[sh.prim0 + k];
                const float ea = exp2_neg(pa.a2 * ar.rr[0]);
                if (k + 1 < nk) {
                    const PrimMx pb = B.prim_mx[sh.prim0 + k + 1];
                    const float eb = exp2_neg(pb.a2 * ar.rr[0]);
                    R0 = fmaf(pb.w, eb, R0);
                    R1 = fmaf(pb.wa, eb, R1);
                }
                R0 = fmaf(pa.w, ea, R0);
                R1 = fmaf(pa.wa, ea, R1);
            }
            const Radial<float> r{R0, R1, 0.f};
            shell_eval_L(sh.L, ar.X[0], ar.Y[0], ar.Z[0], r, chmask, false, [&](int ch, int j, float v) {
                __nv_bfloat16 b0, b1, b2;
                split3(v, b0, b1, b2);
                unsigned char* base = A_s + ch * 3 * A_TILE + amn_off(r0, sh.mcol + j);
                *(__nv_bfloat16*)(base) = b0;
                *(__nv_bfloat16*)(base + A_TILE) = b1;
                *(__nv_bfloat16*)(base + 2 * A_TILE) = b2;
            });
        } else {
            Radial<float> r[2] = {{0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}};
            for (int k = 0; k < nk; ++k) {
                const PrimMx pm = B.prim_mx[sh.prim0 + k];
                const float e0 = exp2_neg(pm.a2 * ar.rr[0]);
                const float e1 = exp2_neg(pm.a2 * ar.rr[1]);
                r[0].R0 = fmaf(pm.w, e0, r[0].R0);
                r[0].R1 = fmaf(pm.wa, e0, r[0].R1);
                r[1].R0 = fmaf(pm.w, e1, r[1].R0);
                r[1].R1 = fmaf(pm.wa, e1, r[1].R1);
            }
            shell_eval2_L(sh.L, ar.X, ar.Y, ar.Z, r, chmask, [&](int ch, int j, float v0, float v1) {
                // v = b0 + b1 + b2 to 2^-24 for both points, each part a packed pair
                const __nv_bfloat162 h0 = __floats2bfloat162_rn(v0, v1);
                const float2 f0 = __bfloat1622float2(h0);
                const float s0 = v0 - f0.x, s1 = v1 - f0.y;
                const __nv_bfloat162 h1 = __floats2bfloat162_rn(s0, s1);
                const float2 f1 = __bfloat1622float2(h1);
                const __nv_bfloat162 h2 = __floats2bfloat162_rn(s0 - f1.x, s1 - f1.y);
                unsigned char* base = A_s + ch * 3 * A_TILE + amn_off(r0, sh.mcol + j);
                *(__nv_bfloat162*)(base) = h0;
                *(__nv_bfloat162*)(base + A_TILE) = h1;
                *(__nv_bfloat162*)(base + 2 * A_TILE) = h2;
            });
        }
        si = sn;
    }
    fence_proxy_async();
    mbar_arrive(S.bar_full + 8 * s);
    ++seq;
}

// FP64 part of the MO values (channel ch: 0 value, 1..3 d/dx, d/dy, d/dz) at a cusp
// point that the tensor-core operand left out: for every shell of the cusp atom, its
// primitives with alpha > alpha_c (orbkit's AO of orbkit/c_grid-based.c:38-71 restricted
// to those primitives, exp in FP64), contracted with C_eff in FP64 for the MOs
// [mo0, mo0 + 8).  Called by the lanes whose point is a cusp point only (not inlined:
// its registers stay out of the epilogue's budget).
constexpr double CUSP_NEGLIGIBLE = 50.0;

// The steep primitives of one cusp atom at the point (X, Y, Z from the nucleus):
// for every shell of the atom with a steep primitive that is not negligible there,
// visit(shell, radial sums) -- FP64 exp, orbkit's AO of orbkit/c_grid-based.c:38-71
// restricted to those primitives.
template <typename Visit>
__device__ __forceinline__ void steep_shells(const MolDesc& D, int a, double rr, Visit&& visit)
{
    const BasisDev& B = D.B;
    const int t1 = __ldg(B.atom_shell_ptr + a + 1);
    for (int t = __ldg(B.atom_shell_ptr + a); t < t1; ++t) {
        const Shell sh = load_shell(B.shells + __ldg(B.atom_shells + t));
        Radial<double> r{0.0, 0.0, 0.0};
        bool any = false;
        for (int q = 0; q < sh.nprim; ++q) {
            const double2 pc = __ldg(B.prim_cusp + sh.prim0 + q);
            // steep primitives only; one whose exponential is below e^-50 (2e-22) at the
            // point adds nothing and is dropped
            if (pc.x <= D.alpha_c || pc.x * rr > CUSP_NEGLIGIBLE) continue;
            const double e = pc.y * exp(-pc.x * rr);
            r.R0 += e;
            r.R1 += pc.x * e;
            any = true;
        }
        if (any && !visit(sh, r)) return;
    }
}

// FP64 part of the MO values (channel ch: 0 value, 1..3 d/dx, d/dy, d/dz) that the
// tensor-core operand left out at a point of a cusp tile: the steep primitives of the
// tile's cusp atoms, contracted with C_eff in FP64 for the MOs [mo0, mo0 + 8).  Used when
// the point has more steep components than a CuspVals holds (not inlined: its
// registers stay out of the epilogue's budget).
__device__ __forceinline__ void cusp_part(const MolDesc& D, const EpiPt& ep, int mo0, int ch, double* out)
{
    const BasisDev& B = D.B;
#pragma unroll
    for (int i = 0; i < 8; ++i) out[i] = 0.0;
    for (int ia = 0; ia < ep.ncusp; ++ia) {
        const int a = ep.atoms[ia];
        const double X = ep.x - __ldg(B.atoms + 4 * a), Y = ep.y - __ldg(B.atoms + 4 * a + 1),
                     Z = ep.z - __ldg(B.atoms + 4 * a + 2);
        steep_shells(D, a, X * X + Y * Y + Z * Z, [&](const Shell& sh, const Radial<double>& r) {
            shell_eval_L(sh.L, X, Y, Z, r, 1u << ch, false, [&](int, int j, double v) {
                const int row = __ldg(B.comp_row + sh.comp0 + j);
                if (row < 0) return;
                const double gv = v * __ldg(B.comp_g + sh.comp0 + j);
                const double* cp = D.ceff + (long long)(sh.cart0 + row) * D.nmo + mo0;
                for (int i = 0; i < 8; ++i)
                    if (mo0 + i < D.nmo) out[i] += __ldg(cp + i) * gv;
            });
            return true;
        });
    }
}

// The steep AO values of the tile's cusp atoms at this point, computed once per tile
// (by the first epilogue that reaches the tile) and contracted per 8-MO group: column
// (listed Cartesian row, -1 for none) and channel values (value, d/dx, d/dy, d/dz) of up
// to MAX_SC canonical components; n = 0: nothing steep is left at the point (the
// density products stay on the double-float path); n = -1: more components than that
// (each group then evaluates them again through cusp_part); n = -2: not prepared yet.
constexpr int MAX_SC = 16;
struct CuspVals {
    int n;
    int col[MAX_SC];
    double v[MAX_SC][4];
};

__device__ __forceinline__ void cusp_prepare(const MolDesc& D, const EpiPt& ep, CuspVals& cz)
{
    const BasisDev& B = D.B;
    cz.n = 0;
    for (int ia = 0; ia < ep.ncusp && cz.n >= 0; ++ia) {
        const int a = ep.atoms[ia];
        const double X = ep.x - __ldg(B.atoms + 4 * a), Y = ep.y - __ldg(B.atoms + 4 * a + 1),
                     Z = ep.z - __ldg(B.atoms + 4 * a + 2);
        steep_shells(D, a, X * X + Y * Y + Z * Z, [&](const Shell& sh, const Radial<double>& r) {
            const int base = cz.n;
            if (base + ncanon(sh.L) > MAX_SC) {
                cz.n = -1;
                return false;
            }
            shell_eval_L(sh.L, X, Y, Z, r, 0xFu, false, [&](int ch, int j, double v) {
                const int row = __ldg(B.comp_row + sh.comp0 + j);
                cz.col[base + j] = row < 0 ? -1 : sh.cart0 + row;
                cz.v[base + j][ch] = row < 0 ? 0.0 : v * __ldg(B.comp_g + sh.comp0 + j);
            });
            cz.n = base + ncanon(sh.L);
            return true;
        });
    }
}

// out[i] = sum over the prepared components of C_eff[mo0 + i][col] x value (channel ch).
__device__ __forceinline__ void cusp_contract(const MolDesc& D, const CuspVals& cz, int mo0, int ch, double* out)
{
#pragma unroll
    for (int i = 0; i < 8; ++i) out[i] = 0.0;
    for (int k = 0; k < cz.n; ++k) {
        const int c = cz.col[k];
        if (c < 0) continue;
        const double gv = cz.v[k][ch];
        const double* cp = D.ceff + (long long)c * D.nmo + mo0;  // 8 consecutive MOs of column c
        for (int i = 0; i < 8; ++i)
            if (mo0 + i < D.nmo) out[i] += __ldg(cp + i) * gv;
    }
}

// Generation threads: the epilogue of one job.  Warp w reads TMEM lanes
// 32 (w % 4) .. (its 32 points) and owns the outputs o (0 = rho, 1..3 = d/dx,
// d/dy, d/dz) with o % E == w / 4 (E = generation warps / 4).  The MOs of the job
// are reduced in double-float FP32 (exact products by FMA, two-sum accumulation,
// about 44 bits), added once per job to the FP64 accumulators (GB300's FP64 pipe
// retires two lanes per clock per SM: one FP64 sum per 8 MOs was a third of the
// epilogue).
template <int E, bool CUSP>
__device__ __forceinline__ void gen_epilogue(const MolDesc& D, int pass, int nksteps, const CtaState& S,
                                             uint32_t& accseq, double (&acc)[4], const EpiPt& ep, CuspVals& cz,
                                             int* status)
{
    const int warp = threadIdx.x >> 5;
    const int q = warp & 3, h = warp >> 2;
    const int npad = D.npad;
    bool own[4];
#pragma unroll
    for (int o = 0; o < 4; ++o) own[o] = (o % E == h) && (o == 0 || D.want_grad);
    if (!mbar_wait(S.bar_acc_full, accseq & 1u, status, S.wait_limit)) *S.abort_flag = 1;
    ++accseq;
    tc_fence_after();
    if ((own[0] || own[1] || own[2] || own[3]) && !warp_aborted(S.abort_flag)) {
        const uint32_t tl = S.tmem + ((uint32_t)(32 * q) << 16);
        const float2* occf = D.occf + pass * npad;
        const float2* occ2f = D.occf + (D.npass + pass) * npad;
        if (CUSP && ep.ncusp > 0 && cz.n == -2) cusp_prepare(D, ep, cz);
        const int nlead = nksteps < 4 ? nksteps : 4;  // leading accumulators written in this job
        int mo_end = D.nmo - pass * npad;
        mo_end = mo_end < npad ? (mo_end + 7) & ~7 : npad;
        DF sacc[4];  // this job's double-float sums of the owned outputs
        for (int m0 = 0; m0 < mo_end; m0 += 8) {
            uint32_t q[5][8];
#pragma unroll
            for (int k = 0; k < 5; ++k) tmem_ld8(tl + k * npad + m0, q[k]);
            tmem_wait_ld5(q);
            float v[8], a1[8], a2[8], a3[8], lo[8];
#pragma unroll
            for (int i = 0; i < 8; ++i) {
                v[i] = __uint_as_float(q[0][i]);
                a1[i] = __uint_as_float(q[1][i]);
                a2[i] = __uint_as_float(q[2][i]);
                a3[i] = __uint_as_float(q[3][i]);
                lo[i] = __uint_as_float(q[4][i]);
            }
            // leading accumulators that no K-step of this job wrote hold another
            // job's sums (or nothing yet): they count as zero
            if (nlead < 4) {
#pragma unroll
                for (int i = 0; i < 8; ++i) {
                    a1[i] = nlead > 1 ? a1[i] : 0.f;
                    a2[i] = nlead > 2 ? a2[i] : 0.f;
                    a3[i] = 0.f;
                }
            }
#pragma unroll
            for (int i = 0; i < 8; ++i) v[i] = ((v[i] + a1[i]) + (a2[i] + a3[i])) + lo[i];
            // a cusp point adds the FP64 part of its atom's steep primitives to every MO
            // and forms its products in FP64 (the TMEM loads above and below stay
            // outside this per-lane branch: they are warp-collective)
            const bool cusp = CUSP && ep.ncusp > 0 && cz.n != 0;
            double cv[8];
            if (cusp) {
                if (cz.n >= 0)
                    cusp_contract(D, cz, pass * npad + m0, 0, cv);
                else
                    cusp_part(D, ep, pass * npad + m0, 0, cv);
            }
            if (own[0]) {
                if (!cusp) {
#pragma unroll
                    for (int i = 0; i < 8; ++i) sacc[0].add(df_mul(__ldg(occf + m0 + i), v[i], v[i]));
                } else {
                    const double* oc = D.occ + pass * npad + m0;
                    for (int i = 0; i < 8; ++i) {
                        const double vf = (double)v[i] + cv[i];
                        acc[0] += oc[i] * (vf * vf);
                    }
                }
            }
#pragma unroll
            for (int o = 1; o < 4; ++o) {
                if (!own[o]) continue;
                uint32_t qd[1][8];
                tmem_ld8(tl + (4 + o) * npad + m0, qd[0]);
                tmem_wait_ld1(qd);
                float vd[8];
#pragma unroll
                for (int i = 0; i < 8; ++i) vd[i] = __uint_as_float(qd[0][i]);
                if (!cusp) {
#pragma unroll
                    for (int i = 0; i < 8; ++i) sacc[o].add(df_mul(__ldg(occ2f + m0 + i), v[i], vd[i]));
                } else {
                    double cd[8];
                    if (cz.n >= 0)
                        cusp_contract(D, cz, pass * npad + m0, o, cd);
                    else
                        cusp_part(D, ep, pass * npad + m0, o, cd);
                    const double* oc2 = D.occ + (D.npass + pass) * npad + m0;
                    for (int i = 0; i < 8; ++i)
                        acc[o] += oc2[i] * (((double)v[i] + cv[i]) * ((double)vd[i] + cd[i]));
                }
            }
        }
#pragma unroll
        for (int o = 0; o < 4; ++o)
            if (own[o]) acc[o] += flt_to_dbl(sacc[o].hi) + flt_to_dbl(sacc[o].lo);
    }
    tc_fence_before();
    mbar_arrive(S.bar_acc_empty);
}

// A job of the generation side: one MO pass of one tile.
struct GenJob {
    uint32_t ord;   // tile ordinal of the CTA
    int pass;
    int nch, nks;   // chunks and K-steps generated so far
    long long p;    // this thread's output point (epilogue row)
    bool valid;
};

// Generation side of the CTA.  Jobs (tile, MO pass) are generated in order; the
// first chunk of the next job (screening its tile first when it starts one) is
// generated before the epilogue of the current job, so the tensor core's tail of a
// job overlaps useful work.  The loop has one call site each for chunk generation
// and the epilogue (both are large inlined bodies: a second copy of either doubles
// the hot instruction footprint of the generation warps).
template <int NTG, int P, bool BATCH, bool CUSP>
__device__ __forceinline__ void gen_role(const CtaState& S, int* status)
{
    constexpr int E = NTG / 128;  // epilogue warps per TMEM lane quarter
    const int warp = threadIdx.x >> 5;
    const int h = warp >> 2;
    uint32_t seq = 0, accseq = 0;
    GenPts<P> gp;
    EpiPt ep, ep_g;  // points of the epilogue's tile and of the generated job's tile
    CuspVals cz;     // the epilogue tile's steep AO values at this thread's cusp point
    cz.n = -2;       // -2: not prepared for the current tile yet
    GenJob g{0u, 0, 0, 0, 0, false}, e = g;  // the job being generated, the job whose epilogue is due
    if (gen_open_tile<P, BATCH, CUSP>(S, 0u, g.p, g.valid, gp, ep, status) < 0) return;
    AtomRun<P> ar;
    int c = next_kept(S.kmask, S.mol[0].B.nmchunk, -1);
    bool due = false, more = true;
    double acc[4] = {0.0, 0.0, 0.0, 0.0};
    for (;;) {
        if (c >= 0) {
            const MolDesc& Dg = S.mol[BATCH ? tbuf(g.ord) : 0];
            const unsigned* km = S.kmask + tbuf(g.ord) * MAX_CHUNKS;
            if (warp_aborted(S.abort_flag)) {
                c = -1;
            } else {
                gen_chunk<NTG, P>(Dg.B, S.nkeep + tbuf(g.ord) * MAX_SHELLS, c, S, seq, ar,
                                  Dg.want_grad ? 0xFu : 0x1u, gp, status);
                ++g.nch;
                g.nks += ksteps_of(km[c]);
                c = next_kept(km, Dg.B.nmchunk, c);
            }
        } else if (!due) {
            // every chunk of job g is out
            const MolDesc& Dg = S.mol[BATCH ? tbuf(g.ord) : 0];
            // single molecule: the tile's screening tables are not read after its last
            // chunk, so the buffer is released now and the tile warp screens ahead during
            // this job's epilogue (a batch releases after the stores: the buffer also holds
            // the molecule's descriptor)
            if (!BATCH && g.pass == Dg.npass - 1) mbar_arrive(S.bar_kfree + 8 * tbuf(g.ord));
            // the next job: the next MO pass of this tile, or pass 0 of a new tile
            GenJob n = g;
            n.pass = g.pass + 1;
            n.nch = n.nks = 0;
            if (n.pass == Dg.npass) {
                n.ord = g.ord + 1;
                n.pass = 0;
                more = gen_open_tile<P, BATCH, CUSP>(S, n.ord, n.p, n.valid, gp, ep_g, status) >= 0;
            }
            e = g;
            due = true;
            if (more) {
                g = n;
                ar = AtomRun<P>();
                c = next_kept(S.kmask + tbuf(g.ord) * MAX_CHUNKS, S.mol[BATCH ? tbuf(g.ord) : 0].B.nmchunk, -1);
            }
        }
        // job e's epilogue once the next job's first chunk is out (or it has none)
        if (due && (g.nch > 0 || c < 0 || !more)) {
            const MolDesc& De = S.mol[BATCH ? tbuf(e.ord) : 0];
            // (nothing to read if none of its chunks reached the tensor core)
            if (e.nch > 0) gen_epilogue<E, CUSP>(De, e.pass, e.nks, S, accseq, acc, ep, cz, status);
            if (e.pass == De.npass - 1) {
                if (e.valid && !*S.abort_flag) {
                    if (0 % E == h) De.rho[e.p] = acc[0];
                    if (De.want_grad) {
#pragma unroll
                        for (int o = 1; o < 4; ++o)
                            if (o % E == h) De.grad[(long long)(o - 1) * De.ld + e.p] = acc[o];
                    }
                }
#pragma unroll
                for (int o = 0; o < 4; ++o) acc[o] = 0.0;
                // this thread is done with the tile's buffer (descriptor, screening tables)
                if (BATCH) mbar_arrive(S.bar_kfree + 8 * tbuf(e.ord));
            }
            due = false;
            if (!more) break;
            if (g.ord != e.ord) {
                ep = ep_g;
                cz.n = -2;
            }
        }
    }
}

// A chunk as the MMA warp needs it, with its molecule's fields copied to registers.
struct MmaItem {
    const uint4* bpack;
    int npad, nmchunk, npass, nch;
    uint32_t ord;  // tile ordinal of the CTA
    int pass, c;
    unsigned km;   // kept columns of the chunk
};

// MMA warp: the next kept chunk after `it` inside its tile, in (pass, chunk) order.
__device__ __forceinline__ bool mma_next_in_tile(const CtaState& S, MmaItem& it)
{
    const unsigned* km = S.kmask + tbuf(it.ord) * MAX_CHUNKS;
    for (;;) {
        ++it.c;
        if (it.c == it.nmchunk) {
            it.c = -1;
            if (++it.pass == it.npass) return false;
            continue;
        }
        const unsigned k = km[it.c];
        if (k != 0u) {
            it.km = k;
            return true;
        }
    }
}

// MMA warp: release the buffer of tile it.ord (unless it.ord is the first to
// open), then open the following tiles (after the generation threads screened
// them) until one has a kept chunk.  False when there are no more tiles.
template <bool BATCH>
__device__ __forceinline__ bool mma_open_next(const CtaState& S, MmaItem& it, bool release, int* status)
{
    const int lane = threadIdx.x & 31;
    for (;;) {
        if (release) {
            __syncwarp();
            if (lane == 0) mbar_arrive(S.bar_kfree + 8 * tbuf(it.ord));
            ++it.ord;
        }
        release = true;
        const int b = tbuf(it.ord);
        if (!mbar_wait(S.bar_screened + 8 * b, tphase(it.ord), status, S.wait_limit)) *S.abort_flag = 1;
        if (S.tile_slot[b] < 0 || *S.abort_flag) return false;
        const MolDesc& D = S.mol[BATCH ? b : 0];
        it.bpack = D.bpack;
        it.npad = D.npad;
        it.nmchunk = D.B.nmchunk;
        it.npass = D.npass;
        it.nch = D.want_grad ? 4 : 1;
        it.pass = 0;
        it.c = -1;
        if (mma_next_in_tile(S, it)) return true;
    }
}

// MMA warp, lane 0: the bulk copy of an item's B block into stage seq % 2 once
// that stage's previous MMAs are complete.  Nothing is issued once the CTA has
// aborted (or if the stage does not free up): returns whether the copy is in
// flight, so that the warp can wait for it before the CTA leaves.
__device__ __forceinline__ bool mma_prefetch_b(const CtaState& S, const MmaItem& it, uint32_t seq, int* status)
{
    const uint32_t s = seq & 1u, u = seq >> 1;
    const int bunits = 3 * it.npad * RUNITS;
    if (u > 0 && !mbar_wait(S.bar_empty + 8 * s, (u - 1) & 1u, status, S.wait_limit)) *S.abort_flag = 1;
    if (*S.abort_flag) return false;
    bulk_load(smem_u32(S.B_s + s * B_STAGE), it.bpack + ((long long)it.pass * it.nmchunk + it.c) * bunits,
              (uint32_t)bunits * 16u, S.bar_bload + 8 * s);
    return true;
}

// One chunk's MMAs from one thread: per issued K-step and channel the six
// (A part, B part) products b0c0 b0c1 b1c0 b0c2 b1c1 b2c0.  The value channel's
// leading product goes to accumulator ks mod 4 (ks: K-step of the job), its five
// corrections to accumulator 4; gradient channel ch takes all six in accumulator
// 4 + ch.  after_first() runs once, after the first issued K-step.  The loops stay
// rolled: the warp shares its SM sub-partition's instruction cache with generation
// warps.
template <typename F>
__device__ __forceinline__ void mma_issue_chunk(uint32_t tmem, int npad, int nch, uint32_t a_lo, uint32_t a_hi,
                                                uint32_t b_lo, uint32_t b_hi, unsigned km, int kq, F&& after_first)
{
    const uint32_t idesc = idesc_bf16(M, npad);
    const uint32_t bpart = (uint32_t)(npad * ROWB) >> 4;
    constexpr uint32_t apart = A_TILE >> 4;
    const bool kon0 = (km & 0xFFFFu) != 0u, kon1 = (km >> 16) != 0u;
    bool first = true;
#pragma unroll 1
    for (int k = 0; k < KC / 16; ++k) {
        if (!(k == 0 ? kon0 : kon1)) continue;  // all 16 columns screened
        const int ks = kq + (k == 1 && kon0);
        const uint32_t f0 = ks > 0;
        const uint32_t bk = b_lo + (uint32_t)((k * 32) >> 4);
#pragma unroll 1
        for (int ch = 0; ch < nch; ++ch) {
            const uint32_t a0 = a_lo + (uint32_t)((ch * 3 * A_TILE + k * 4096) >> 4);
            const uint32_t dc = tmem + (uint32_t)((4 + ch) * npad);  // corrections / gradient
            const uint32_t dl = ch == 0 ? tmem + (uint32_t)((ks & 3) * npad) : dc;
            const uint32_t fl = ch == 0 ? (uint32_t)(ks >= 4) : f0;
            const uint32_t f1 = ch == 0 ? f0 : 1u;
            mma_bf16_w(dl, a0, a_hi, bk, b_hi, idesc, fl);
            mma_bf16_w(dc, a0, a_hi, bk + bpart, b_hi, idesc, f1);
            mma_bf16_w(dc, a0 + apart, a_hi, bk, b_hi, idesc, 1u);
            mma_bf16_w(dc, a0, a_hi, bk + 2 * bpart, b_hi, idesc, 1u);
            mma_bf16_w(dc, a0 + apart, a_hi, bk + bpart, b_hi, idesc, 1u);
            mma_bf16_w(dc, a0 + 2 * apart, a_hi, bk, b_hi, idesc, 1u);
        }
        if (first) after_first();
        first = false;
    }
}

// MMA side of the CTA (the last warp): for every kept chunk in order, the column
// mask applied to its B block, then 48 MMAs (12 without gradient) from lane 0 once
// the generation threads filled the stage; the next chunk's B block is requested
// halfway through, when the stage it goes to has been consumed.
template <bool BATCH>
__device__ __forceinline__ void mma_role(const CtaState& S, int* status)
{
    const int lane = threadIdx.x & 31;
    uint32_t seq = 0, accseq = 0;
    MmaItem cur;
    cur.ord = 0;
    // lane 0: sequence number of a bulk copy in flight that no wait has seen land
    // (-1: none), and whether any MMA was issued -- both drained before the CTA leaves
    long long pend = -1;
    bool issued = false;
    bool have = mma_open_next<BATCH>(S, cur, false, status);
    if (have && lane == 0 && mma_prefetch_b(S, cur, seq, status)) pend = seq;
    int kq = 0;  // K-steps issued in the current job
    // (loop exits are decided by lane 0 and broadcast: the warp leaves together)
    while (__shfl_sync(0xffffffffu, (int)(have && !*S.abort_flag), 0)) {
        const uint32_t s = seq & 1u, u = seq >> 1;
        unsigned char* B_s = S.B_s + s * B_STAGE;
        const int npad = cur.npad;
        const bool landed = mbar_wait(S.bar_bload + 8 * s, u & 1u, status, S.wait_limit);
        if (!__all_sync(0xffffffffu, landed)) {
            *S.abort_flag = 1;
            break;
        }
        if (pend == (long long)seq) pend = -1;
        const int bunits = 3 * npad * RUNITS;
        // columns of screened shells are zeroed.  Lane l touches the 16-byte units
        // l, l + 32, ...: rows n = l / 4 (mod 8) of every part, physical unit l % 4, so
        // with rows of 4 units and the 64-byte swizzle (unit ^ (n >> 1) % 4) always the
        // same logical 8-column group
        const unsigned m8 = (cur.km >> (8 * ((lane & 3) ^ ((lane >> 3) & 3)))) & 0xFFu;
        if (m8 != 0xFFu) {
            unsigned keep[4];
#pragma unroll
            for (int t = 0; t < 4; ++t)
                keep[t] = ((m8 >> (2 * t)) & 1u ? 0x0000FFFFu : 0u) | ((m8 >> (2 * t + 1)) & 1u ? 0xFFFF0000u : 0u);
            // bunits is a multiple of 192: six units per lane at a time, loads first
            uint4* bu = (uint4*)B_s + lane;
            for (int i = 0; i < bunits; i += 192) {
                uint4 v[6];
#pragma unroll
                for (int j = 0; j < 6; ++j) v[j] = bu[i + 32 * j];
#pragma unroll
                for (int j = 0; j < 6; ++j)
                    bu[i + 32 * j] = make_uint4(v[j].x & keep[0], v[j].y & keep[1], v[j].z & keep[2], v[j].w & keep[3]);
            }
            fence_proxy_async();
        }
        MmaItem nxt = cur;
        const bool in_tile = mma_next_in_tile(S, nxt);  // the next chunk if it is in this tile
        __syncwarp();
        if (lane == 0) {
            // the previous job's accumulators must have been read before they are overwritten
            if (kq == 0 && accseq > 0 && !mbar_wait(S.bar_acc_empty, (accseq - 1) & 1u, status, S.wait_limit))
                *S.abort_flag = 1;
            if (!mbar_wait(S.bar_full + 8 * s, u & 1u, status, S.wait_limit)) *S.abort_flag = 1;
            tc_fence_after();
            if (!*S.abort_flag) {
                const uint64_t ad = adesc_mn(smem_u32(S.A_s + s * A_STAGE)), bd = sdesc(smem_u32(B_s));
                // the next chunk's B block is requested once the first K-step is out
                auto prefetch = [&]() {
                    if (in_tile && mma_prefetch_b(S, nxt, seq + 1, status)) pend = seq + 1;
                };
                mma_issue_chunk(S.tmem, npad, cur.nch, (uint32_t)ad, (uint32_t)(ad >> 32), (uint32_t)bd,
                                (uint32_t)(bd >> 32), cur.km, kq, prefetch);
                issued = true;
                mma_commit(S.bar_empty + 8 * s);
            } else {
                mbar_arrive(S.bar_empty + 8 * s);
            }
            if (!in_tile || nxt.pass != cur.pass) {
                // last chunk of the job: hand the accumulators to the epilogue
                if (!*S.abort_flag)
                    mma_commit(S.bar_acc_full);
                else
                    mbar_arrive(S.bar_acc_full);
            }
        }
        __syncwarp();
        ++seq;
        kq += ksteps_of(cur.km);
        if (!in_tile || nxt.pass != cur.pass) {
            ++accseq;
            kq = 0;
        }
        have = in_tile;
        if (!in_tile) {
            // leave the tile once its last chunk's MMAs are issued; the next tile's
            // first B block is requested as soon as the tile is open
            have = mma_open_next<BATCH>(S, nxt, true, status);
            if (have && lane == 0 && mma_prefetch_b(S, nxt, seq, status)) pend = seq;
        }
        cur = nxt;
    }
    // before the CTA leaves (normally or after an expired wait): the bulk copy still
    // in flight lands and every issued MMA completes, so that no asynchronous write
    // reaches shared or tensor memory after the teardown
    __syncwarp();
    if (lane == 0) {
        if (pend >= 0) mbar_drain(S.bar_bload + 8 * (uint32_t)(pend & 1), (uint32_t)(pend >> 1) & 1u);
        if (issued) {
            mma_commit(S.bar_drain);
            mbar_drain(S.bar_drain, 0);
        }
    }
    __syncwarp();
}

// CTA set-up shared by the kernels: shared-memory carve-up, A stages zeroed
// (columns of screened shells keep stale but finite values, multiplied by zeroed B
// columns), mbarriers, TMEM allocation.  NTT threads in all, NTG of them generate.
template <int NTT, int NTG>
__device__ __forceinline__ CtaState cta_setup(unsigned char* smem, MolDesc* mol, uint32_t tm_cols, long long wait_limit)
{
    const int tid = threadIdx.x, warp = tid >> 5;
    CtaState S;
    S.A_s = smem;
    S.B_s = smem + NSTAGE * A_STAGE;
    S.kmask = (unsigned*)(S.B_s + NSTAGE * B_STAGE);
    // full[2], empty[2], bload[2], acc full, acc empty, screened[NBUF], kfree[NBUF], drain
    uint64_t* bar = (uint64_t*)(S.kmask + NBUF * MAX_CHUNKS);
    S.tile_slot = (long long*)(bar + 9 + 2 * NBUF);
    uint32_t* tmem_slot = (uint32_t*)(S.tile_slot + NBUF);
    S.abort_flag = (int*)(tmem_slot + 1);
    S.nkeep = (unsigned char*)(S.abort_flag + 1);
    S.cusp_atoms = (int*)(S.nkeep + NBUF * MAX_SHELLS);
    S.mol = mol;
    S.bar_full = smem_u32(bar);
    S.bar_empty = smem_u32(bar + 2);
    S.bar_bload = smem_u32(bar + 4);
    S.bar_acc_full = smem_u32(bar + 6);
    S.bar_acc_empty = smem_u32(bar + 7);
    S.bar_screened = smem_u32(bar + 8);
    S.bar_kfree = smem_u32(bar + 8 + NBUF);
    S.bar_drain = smem_u32(bar + 8 + 2 * NBUF);
    S.wait_limit = wait_limit;
    for (int i = tid; i < NSTAGE * A_STAGE / 16; i += NTT) ((uint4*)S.A_s)[i] = make_uint4(0, 0, 0, 0);
    if (tid == 0) {
        for (int s = 0; s < NSTAGE; ++s) {
            mbar_init(S.bar_full + 8 * s, NTG);
            mbar_init(S.bar_empty + 8 * s, 1);
            mbar_init(S.bar_bload + 8 * s, 1);
        }
        mbar_init(S.bar_acc_full, 1);
        mbar_init(S.bar_acc_empty, NTG);
        for (int b = 0; b < NBUF; ++b) {
            mbar_init(S.bar_screened + 8 * b, 32);     // the tile warp
            mbar_init(S.bar_kfree + 8 * b, NTG + 1);   // every generation thread and the MMA warp
        }
        mbar_init(S.bar_drain, 1);
        *S.abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(tm_cols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    fence_proxy_async();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    S.tmem = *tmem_slot;
    return S;
}

// bytes of dynamic shared memory of the mixed kernels (1 KB alignment slack included)
constexpr size_t SMEM_BYTES = 1024 + NSTAGE * (A_STAGE + B_STAGE) + 4 * NBUF * MAX_CHUNKS + (9 + 2 * NBUF) * 8 +
                              NBUF * 8 + 4 + 4 + NBUF * MAX_SHELLS + NBUF * (1 + NCA) * 4 + 64;
static_assert(SMEM_BYTES + NBUF * sizeof(MolDesc) <= 232448, "mixed kernel shared memory above the 227 KB per-CTA limit");
static_assert(KC == 32, "column masks are 32-bit and operand rows one 64-byte swizzle row");
static_assert(sizeof(MolDesc) % 16 == 0, "descriptors are copied in 16-byte units");

__device__ __forceinline__ void cta_teardown(const CtaState& S, uint32_t tm_cols)
{
    tc_fence_before();
    __syncthreads();
    if ((threadIdx.x >> 5) == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(S.tmem), "r"(tm_cols));
}

__host__ __device__ inline uint32_t tmem_cols_for(int npad)
{
    const int n = 8 * npad;
    return n <= 32 ? 32 : n <= 64 ? 64 : n <= 128 ? 128 : n <= 256 ? 256 : 512;
}

// Tiles of a grid: 4 x 4 x 8 bricks when the call covers a whole regular grid,
// else runs of 128 flattened points.
inline void tiling(const Grid& g, MolDesc& D)
{
    D.brick = g.regular && g.offset == 0 && g.npts == (long long)g.nx * g.ny * g.nz;
    if (D.brick) {
        const long long nbx = (g.nx + 3) / 4;
        D.nby = (g.ny + 3) / 4;
        D.nbz = (g.nz + 7) / 8;
        D.ntiles = nbx * D.nby * D.nbz;
    } else {
        D.nby = D.nbz = 0;
        D.ntiles = (g.npts + M - 1) / M;
    }
}

// Descriptor of one molecule's call (host side).
inline void make_desc(MolDesc& D, const BasisDev& B, const Grid& g, const void* bpack, const double* occ, int npass,
                      int npad, int nmo, int want_grad, double* rho, double* grad, long long ld,
                      const short* near = nullptr, const double* ceff = nullptr, double alpha_c = 0.0)
{
    memset(&D, 0, sizeof(D));
    D.B = B;
    D.g = g;
    D.bpack = (const uint4*)bpack;
    D.occ = occ;
    D.occf = (const float2*)(occ + 2 * npass * npad);
    D.rho = rho;
    D.grad = want_grad ? grad : nullptr;
    D.ld = ld;
    D.tile0 = 0;
    D.npass = npass;
    D.npad = npad;
    D.nmo = nmo;
    D.want_grad = want_grad;
    D.near = ceff ? near : nullptr;
    D.ceff = ceff;
    D.alpha_c = alpha_c;
    tiling(g, D);
}

// Dynamic shared memory: aligned to 1024 bytes by hand (SMEM_BYTES holds the slack);
// declaring it __align__(1024) would round the static part (the molecule descriptors)
// up to a multiple of 1 KB and push the total past the 227 KB per-CTA limit.
extern __shared__ __align__(16) unsigned char mx_smem_raw[];

// Single molecule: its descriptor is copied to shared memory once.
// Threads of a CTA: NTG generation threads, the MMA warp and the tile warp.
__host__ __device__ constexpr int cta_threads(int ntg) { return ntg + 64; }

template <int NTG, int PP, bool CUSP>
__global__ void __launch_bounds__(cta_threads(NTG), 1) rho_mixed_kernel(const __grid_constant__ Params P)
{
    __shared__ MolDesc mol[1];
    unsigned char* smem = (unsigned char*)(((uintptr_t)mx_smem_raw + 1023) & ~(uintptr_t)1023);
    if (threadIdx.x < sizeof(MolDesc) / 16) ((uint4*)mol)[threadIdx.x] = ((const uint4*)&P.D)[threadIdx.x];
    const uint32_t tm_cols = tmem_cols_for(P.D.npad);
    CtaState S = cta_setup<cta_threads(NTG), NTG>(smem, mol, tm_cols, P.wait_limit);
    TileFeed F;
    F.counter = P.counter;
    F.ntiles = P.D.ntiles;
    F.descs = nullptr;
    F.nmol = 1;
    F.grab = 1;
    if (threadIdx.x < NTG)
        gen_role<NTG, PP, false, CUSP>(S, P.status);
    else if (threadIdx.x < NTG + 32)
        mma_role<false>(S, P.status);
    else
        tile_role<NTG * PP / 128, false, CUSP>(F, S, P.status);
    cta_teardown(S, tm_cols);
}

// Batched launch: one persistent CTA per SM; warp 0 takes `grab` consecutive
// tiles of the concatenated tile numbering at a time from a global counter
// (zeroed before the launch), finds each tile's molecule by binary search over
// tile0 and copies its descriptor into the tile's buffer.
struct BatchParams {
    const MolDesc* descs;  // nmol, ascending tile0
    int nmol;
    int grab;
    long long total_tiles;
    unsigned long long* counter;
    int* status;
    long long wait_limit;
};

template <int NTG, int PP, bool CUSP>
__global__ void __launch_bounds__(cta_threads(NTG), 1) rho_mixed_batch_kernel(const BatchParams P)
{
    __shared__ MolDesc mol[NBUF];
    unsigned char* smem = (unsigned char*)(((uintptr_t)mx_smem_raw + 1023) & ~(uintptr_t)1023);
    CtaState S = cta_setup<cta_threads(NTG), NTG>(smem, mol, 512, P.wait_limit);
    TileFeed F;
    F.counter = P.counter;
    F.ntiles = P.total_tiles;
    F.descs = P.descs;
    F.nmol = P.nmol;
    F.grab = P.grab;
    if (threadIdx.x < NTG)
        gen_role<NTG, PP, true, CUSP>(S, P.status);
    else if (threadIdx.x < NTG + 32)
        mma_role<true>(S, P.status);
    else
        tile_role<NTG * PP / 128, true, CUSP>(F, S, P.status);
    cta_teardown(S, 512);
}

// Split C_eff (nmo x ncart, FP64) times the columns' angular norms into three
// BF16 parts in the B operand layout:
// bpack[pass][chunk][part] is an npad x 32 K-major SWIZZLE_64B tile whose column
// kk holds the coefficient of the listed Cartesian AO feeding mixed column kk.
__global__ void pack_b_kernel(const double* __restrict__ C, int nmo, int ncart, const int* __restrict__ mcol_cart,
                              const double* __restrict__ mcol_g, int nmchunk, int npass, int npad,
                              __nv_bfloat16* __restrict__ bpack)
{
    const long long total = (long long)npass * nmchunk * npad * KC;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const int kk = (int)(i % KC);
        const int n = (int)((i / KC) % npad);
        const int c = (int)((i / ((long long)KC * npad)) % nmchunk);
        const int pass = (int)(i / ((long long)KC * npad * nmchunk));
        const int mo = pass * npad + n;
        const int cart = mcol_cart[c * KC + kk];
        double v = (mo < nmo && cart >= 0) ? C[(long long)mo * ncart + cart] * mcol_g[c * KC + kk] : 0.0;
        const __nv_bfloat16 h0 = __double2bfloat16(v);
        const double r1 = v - (double)__bfloat162float(h0);
        const __nv_bfloat16 h1 = __double2bfloat16(r1);
        const double r2 = r1 - (double)__bfloat162float(h1);
        const __nv_bfloat16 h2 = __double2bfloat16(r2);
        const uint32_t off = sw64_off(n, kk);
        unsigned char* blk = (unsigned char*)bpack + ((long long)pass * nmchunk + c) * (3ll * npad * ROWB);
        *(__nv_bfloat16*)(blk + off) = h0;
        *(__nv_bfloat16*)(blk + npad * ROWB + off) = h1;
        *(__nv_bfloat16*)(blk + 2 * npad * ROWB + off) = h2;
    }
}

// C_eff (nmo x ncart) -> its transpose (ncart x nmo) for the FP64 cusp part.
__global__ void transpose_kernel(const double* __restrict__ C, int nmo, int ncart, double* __restrict__ T)
{
    const long long n = (long long)nmo * ncart;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const int c = (int)(i / nmo), m = (int)(i - (long long)c * nmo);
        T[i] = C[(long long)m * ncart + c];
    }
}

// out[0 .. total): occupations (zero padded); out[total .. 2 total): twice them;
// then the same 2 total values as double-float (hi, lo) pairs.
__global__ void pack_occ_kernel(const double* __restrict__ occ, int nmo, int total, double* __restrict__ out)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < total) {
        const double o = i < nmo ? occ[i] : 0.0;
        out[i] = o;
        out[total + i] = 2.0 * o;
        float2* f = (float2*)(out + 2 * total);
        const float oh = (float)o, o2h = (float)(2.0 * o);
        f[i] = make_float2(oh, (float)(o - (double)oh));
        f[total + i] = make_float2(o2h, (float)(2.0 * o - (double)o2h));
    }
}

}  // namespace mx
}  // namespace okg

using namespace okg;

namespace okg {
namespace mx {
// Shared-memory attribute of every instantiation (idempotent, called at set-up).
// Generation layouts {generation threads per CTA, grid points per generation
// thread} with a kernel instantiation each.
constexpr int GEN_LAYOUTS[][2] = {{256, 1}, {384, 1}, {512, 1}, {256, 2}, {384, 2}};
constexpr int NLAYOUT = (int)(sizeof(GEN_LAYOUTS) / sizeof(GEN_LAYOUTS[0]));

constexpr int LAYOUT_DEFAULT = 1;  // 384 generation threads, one point each

inline int layout_index(int threads, int points)
{
    for (int i = 0; i < NLAYOUT; ++i)
        if (GEN_LAYOUTS[i][0] == threads && GEN_LAYOUTS[i][1] == points) return i;
    return -1;
}

template <int NTG, int PP>
static cudaError_t configure_one()
{
    const int sm = (int)SMEM_BYTES;
    cudaError_t e =
        cudaFuncSetAttribute(rho_mixed_kernel<NTG, PP, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(rho_mixed_batch_kernel<NTG, PP, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 sm);
    // the FP64 cusp variants exist for one point per generation thread
    if constexpr (PP == 1) {
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(rho_mixed_kernel<NTG, PP, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm);
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(rho_mixed_batch_kernel<NTG, PP, true>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, sm);
    }
    return e;
}

// Shared-memory attribute of every instantiation (idempotent, called at set-up).
static cudaError_t configure_kernels()
{
    cudaError_t e = configure_one<256, 1>();
    if (e == cudaSuccess) e = configure_one<384, 1>();
    if (e == cudaSuccess) e = configure_one<512, 1>();
    if (e == cudaSuccess) e = configure_one<256, 2>();
    if (e == cudaSuccess) e = configure_one<384, 2>();
    return e;
}

// cusp: the FP64 cusp variant (layouts with one point per generation thread only;
// the callers check)
static void launch_single(int layout, bool cusp, unsigned grid, cudaStream_t st, const Params& P)
{
    if (cusp) {
        switch (layout) {
        case 0: rho_mixed_kernel<256, 1, true><<<grid, cta_threads(256), SMEM_BYTES, st>>>(P); break;
        case 2: rho_mixed_kernel<512, 1, true><<<grid, cta_threads(512), SMEM_BYTES, st>>>(P); break;
        default: rho_mixed_kernel<384, 1, true><<<grid, cta_threads(384), SMEM_BYTES, st>>>(P); break;
        }
        return;
    }
    switch (layout) {
    case 0: rho_mixed_kernel<256, 1, false><<<grid, cta_threads(256), SMEM_BYTES, st>>>(P); break;
    case 2: rho_mixed_kernel<512, 1, false><<<grid, cta_threads(512), SMEM_BYTES, st>>>(P); break;
    case 3: rho_mixed_kernel<256, 2, false><<<grid, cta_threads(256), SMEM_BYTES, st>>>(P); break;
    case 4: rho_mixed_kernel<384, 2, false><<<grid, cta_threads(384), SMEM_BYTES, st>>>(P); break;
    default: rho_mixed_kernel<384, 1, false><<<grid, cta_threads(384), SMEM_BYTES, st>>>(P); break;
    }
}

static void launch_batch(int layout, bool cusp, unsigned grid, cudaStream_t st, const BatchParams& P)
{
    if (cusp) {
        switch (layout) {
        case 0: rho_mixed_batch_kernel<256, 1, true><<<grid, cta_threads(256), SMEM_BYTES, st>>>(P); break;
        case 2: rho_mixed_batch_kernel<512, 1, true><<<grid, cta_threads(512), SMEM_BYTES, st>>>(P); break;
        default: rho_mixed_batch_kernel<384, 1, true><<<grid, cta_threads(384), SMEM_BYTES, st>>>(P); break;
        }
        return;
    }
    switch (layout) {
    case 0: rho_mixed_batch_kernel<256, 1, false><<<grid, cta_threads(256), SMEM_BYTES, st>>>(P); break;
    case 2: rho_mixed_batch_kernel<512, 1, false><<<grid, cta_threads(512), SMEM_BYTES, st>>>(P); break;
    case 3: rho_mixed_batch_kernel<256, 2, false><<<grid, cta_threads(256), SMEM_BYTES, st>>>(P); break;
    case 4: rho_mixed_batch_kernel<384, 2, false><<<grid, cta_threads(384), SMEM_BYTES, st>>>(P); break;
    default: rho_mixed_batch_kernel<384, 1, false><<<grid, cta_threads(384), SMEM_BYTES, st>>>(P); break;
    }
}

inline bool layout_has_cusp(int layout) { return GEN_LAYOUTS[layout][1] == 1; }
}  // namespace mx
}  // namespace okg

struct okg_mixed_plan {
    const okg_basis* basis;
    int nmo, npad, npass;
    void* block;       // bpack | occ | status
    size_t bpack_bytes;
    __nv_bfloat16* bpack;
    double* occ;
    int* status;
    int sm_count;
    size_t smem;
    int layout;  // index into GEN_LAYOUTS (generation threads, points per thread)
    long long wait_limit;  // polls per bounded device wait (WAIT_LIMIT by default)
    double* ceff;          // C_eff in FP64, transposed (ncart x nmo), for the cusp points
    const short* near;     // caller's cusp-atom index per point, or null (no cusp treatment)
    double alpha_c;        // primitives with alpha > alpha_c are FP64 at cusp points
};

extern "C" int okg_mixed_plan_create_tiled(const okg_basis* b, int nmo, int n_max, okg_mixed_plan** out);

extern "C" int okg_mixed_plan_create(const okg_basis* b, int nmo, okg_mixed_plan** out)
{
    return okg_mixed_plan_create_tiled(b, nmo, mx::NMAX, out);
}

extern "C" int okg_mixed_plan_create_tiled(const okg_basis* b, int nmo, int n_max, okg_mixed_plan** out)
{
    if (!out || !b || nmo <= 0) return set_error(OKG_ERR_ARG, "okg_mixed_plan_create: NULL basis/out or nmo <= 0");
    if (n_max < 16 || n_max > mx::NMAX || n_max % 16)
        return set_error(OKG_ERR_ARG, "okg_mixed_plan_create_tiled: n_max must be 16, 32, 48 or 64");
    *out = nullptr;
    int dev = 0, major = 0, minor = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev);
    cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (major != 10 || minor != 3) return set_error(OKG_ERR_DEVICE, "okg_mixed_plan_create: needs an sm_103 GPU");
    if (b->dev.nshell > mx::MAX_SHELLS || b->dev.nmchunk > mx::MAX_CHUNKS)
        return set_error(OKG_ERR_UNSUPPORTED, "okg_mixed_plan_create: more than 2048 shells or 192 column chunks");
    if (b->dev.max_nprim > mx::MAX_PRIM)
        return set_error(OKG_ERR_UNSUPPORTED, "okg_mixed_plan_create: a shell with more than 31 primitives");
    okg_mixed_plan* p = (okg_mixed_plan*)calloc(1, sizeof(okg_mixed_plan));
    if (!p) return set_error(OKG_ERR_ALLOC, "okg_mixed_plan_create: host allocation");
    b->mixed_locked = 1;  // the coefficient tiles follow the basis's column order from now on
    p->basis = b;
    p->nmo = nmo;
    p->npass = (nmo + n_max - 1) / n_max;
    const int per = (nmo + p->npass - 1) / p->npass;
    p->npad = (per + 15) / 16 * 16;
    p->bpack_bytes = (size_t)p->npass * b->dev.nmchunk * 3 * p->npad * mx::ROWB;
    const size_t occ_off = (p->bpack_bytes + 255) & ~(size_t)255;
    const size_t st_off = occ_off + (((size_t)4 * p->npass * p->npad * 8 + 255) & ~(size_t)255);
    const size_t ceff_off = st_off + 256;
    cudaError_t e = cudaMalloc(&p->block, ceff_off + (size_t)nmo * b->dev.ncart * sizeof(double));
    if (e != cudaSuccess) {
        free(p);
        return cuda_status(e, "okg_mixed_plan_create: cudaMalloc");
    }
    p->bpack = (__nv_bfloat16*)p->block;
    p->occ = (double*)((char*)p->block + occ_off);
    p->status = (int*)((char*)p->block + st_off);
    p->ceff = (double*)((char*)p->block + ceff_off);
    p->near = nullptr;
    p->alpha_c = 0.0;
    cudaMemset(p->status, 0, sizeof(int));
    p->sm_count = sms;
    p->smem = mx::SMEM_BYTES;
    p->layout = mx::LAYOUT_DEFAULT;
    p->wait_limit = mx::WAIT_LIMIT;
    e = mx::configure_kernels();
    if (e != cudaSuccess) {
        cudaFree(p->block);
        free(p);
        return cuda_status(e, "okg_mixed_plan_create: shared memory attribute");
    }
    *out = p;
    return OKG_OK;
}

extern "C" int okg_mixed_plan_set_threads(okg_mixed_plan* p, int threads)
{
    if (!p || (threads != 256 && threads != 384 && threads != 512))
        return set_error(OKG_ERR_ARG, "okg_mixed_plan_set_threads: threads must be 256, 384 or 512");
    p->layout = mx::layout_index(threads, 1);
    return OKG_OK;
}

extern "C" int okg_mixed_plan_set_generation(okg_mixed_plan* p, int threads, int points_per_thread)
{
    const int l = mx::layout_index(threads, points_per_thread);
    if (!p || l < 0)
        return set_error(OKG_ERR_ARG, "okg_mixed_plan_set_generation: (threads, points) must be (256|384|512, 1) or "
                                      "(256|384, 2)");
    p->layout = l;
    return OKG_OK;
}

extern "C" int okg_mixed_plan_set_wait_limit(okg_mixed_plan* p, long long polls)
{
    if (!p || polls < 1) return set_error(OKG_ERR_ARG, "okg_mixed_plan_set_wait_limit: NULL plan or polls < 1");
    p->wait_limit = polls;
    return OKG_OK;
}

extern "C" int okg_mixed_plan_destroy(okg_mixed_plan* p)
{
    if (!p) return OKG_OK;
    cudaError_t e = cudaFree(p->block);
    free(p);
    return cuda_status(e, "okg_mixed_plan_destroy");
}

extern "C" int okg_mixed_set_coeffs(okg_mixed_plan* p, const double* d_coeff, const double* d_occ, okg_stream stream)
{
    if (!p || !d_coeff || !d_occ) return set_error(OKG_ERR_ARG, "okg_mixed_set_coeffs: NULL argument");
    cudaStream_t st = (cudaStream_t)stream;
    const BasisDev& B = p->basis->dev;
    mx::pack_b_kernel<<<p->sm_count * 4, 256, 0, st>>>(d_coeff, p->nmo, B.ncart, B.mcol_cart, B.mcol_g, B.nmchunk, p->npass,
                                                       p->npad, p->bpack);
    const int total = p->npass * p->npad;
    mx::pack_occ_kernel<<<(total + 127) / 128, 128, 0, st>>>(d_occ, p->nmo, total, p->occ);
    mx::transpose_kernel<<<p->sm_count * 4, 256, 0, st>>>(d_coeff, p->nmo, B.ncart, p->ceff);
    return cuda_status(cudaGetLastError(), "okg_mixed_set_coeffs");
}

extern "C" int okg_mixed_plan_set_cusp(okg_mixed_plan* p, const int16_t* d_near, double alpha_c)
{
    if (!p || alpha_c < 0.0) return set_error(OKG_ERR_ARG, "okg_mixed_plan_set_cusp: NULL plan or alpha_c < 0");
    p->near = (const short*)d_near;
    p->alpha_c = alpha_c;
    return OKG_OK;
}

extern "C" int okg_rho_mixed(okg_mixed_plan* p, const okg_grid* gr, int want_grad, double* d_rho, double* d_grad,
                             int64_t ld, okg_stream stream)
{
    if (!p || !gr || !d_rho || (want_grad && !d_grad)) return set_error(OKG_ERR_ARG, "okg_rho_mixed: NULL argument");
    Grid g;
    g.x = gr->d_x;
    g.y = gr->d_y;
    g.z = gr->d_z;
    g.npts = gr->npts;
    g.offset = gr->offset;
    g.nx = gr->nx;
    g.ny = gr->ny;
    g.nz = gr->nz;
    g.regular = gr->regular;
    if (g.npts < 0 || !g.x || !g.y || !g.z) return set_error(OKG_ERR_ARG, "okg_rho_mixed: bad grid");
    if (g.regular && (g.nx <= 0 || g.ny <= 0 || g.nz <= 0 || g.offset < 0 ||
                      g.offset + g.npts > (long long)g.nx * g.ny * g.nz))
        return set_error(OKG_ERR_ARG, "okg_rho_mixed: regular grid range outside Nx*Ny*Nz");
    if (g.npts == 0) return OKG_OK;
    if (ld < g.npts) return set_error(OKG_ERR_ARG, "okg_rho_mixed: ld < npts");
    mx::Params P;
    mx::make_desc(P.D, p->basis->dev, g, p->bpack, p->occ, p->npass, p->npad, p->nmo, want_grad, d_rho, d_grad, ld,
                  p->near, p->ceff, p->alpha_c);
    P.status = p->status;
    P.counter = (unsigned long long*)((char*)p->status + 64);
    P.wait_limit = p->wait_limit;
    {
        cudaError_t e0 = cudaMemsetAsync(P.counter, 0, sizeof(unsigned long long), (cudaStream_t)stream);
        if (e0 != cudaSuccess) return cuda_status(e0, "okg_rho_mixed: counter reset");
    }
    const bool cusp = P.D.near != nullptr;
    if (cusp && !mx::layout_has_cusp(p->layout))
        return set_error(OKG_ERR_UNSUPPORTED, "okg_rho_mixed: the FP64 cusp points need one point per generation thread");
    const long long grid = P.D.ntiles < p->sm_count ? P.D.ntiles : p->sm_count;
    mx::launch_single(p->layout, cusp, (unsigned)grid, (cudaStream_t)stream, P);
    return cuda_status(cudaGetLastError(), "okg_rho_mixed launch");
}

struct okg_batch {
    int nmol;
    void* block;              // descriptors | counter | status
    mx::MolDesc* d_descs;
    unsigned long long* d_counter;
    int* d_status;
    long long total_tiles;
    int sm_count;
    int grab;
    int ctas;
    size_t smem;
    int layout;
    bool cusp;  // some molecule's plan has FP64 cusp points
};

extern "C" int okg_batch_create(int nmol, okg_mixed_plan* const* plans, const okg_grid* grids, double* const* d_rho,
                                double* const* d_grad, const int64_t* ld, int want_grad, okg_batch** out)
{
    if (!out || nmol <= 0 || !plans || !grids || !d_rho || !ld || (want_grad && !d_grad))
        return set_error(OKG_ERR_ARG, "okg_batch_create: NULL argument or nmol <= 0");
    *out = nullptr;
    std::vector<mx::MolDesc> descs(nmol);
    long long tile0 = 0;
    int sms = 0;
    bool any_cusp = false;
    for (int m = 0; m < nmol; ++m) {
        const okg_mixed_plan* p = plans[m];
        const okg_grid* gr = &grids[m];
        if (!p || !d_rho[m] || (want_grad && !d_grad[m]) || gr->npts < 0 || !gr->d_x || !gr->d_y || !gr->d_z)
            return set_error(OKG_ERR_ARG, "okg_batch_create: molecule with NULL plan, grid or output");
        if (gr->regular && (gr->nx <= 0 || gr->ny <= 0 || gr->nz <= 0 || gr->offset < 0 ||
                            gr->offset + gr->npts > (long long)gr->nx * gr->ny * gr->nz))
            return set_error(OKG_ERR_ARG, "okg_batch_create: regular grid range outside Nx*Ny*Nz");
        if (ld[m] < gr->npts) return set_error(OKG_ERR_ARG, "okg_batch_create: ld < npts");
        mx::MolDesc& D = descs[m];
        Grid g;
        g.x = gr->d_x;
        g.y = gr->d_y;
        g.z = gr->d_z;
        g.npts = gr->npts;
        g.offset = gr->offset;
        g.nx = gr->nx;
        g.ny = gr->ny;
        g.nz = gr->nz;
        g.regular = gr->regular;
        mx::make_desc(D, p->basis->dev, g, p->bpack, p->occ, p->npass, p->npad, p->nmo, want_grad, d_rho[m],
                      want_grad ? d_grad[m] : nullptr, ld[m], p->near, p->ceff, p->alpha_c);
        D.tile0 = tile0;
        tile0 += D.ntiles;
        sms = p->sm_count;
        any_cusp = any_cusp || D.near != nullptr;
    }
    okg_batch* b = (okg_batch*)calloc(1, sizeof(okg_batch));
    if (!b) return set_error(OKG_ERR_ALLOC, "okg_batch_create: host allocation");
    const size_t dbytes = sizeof(mx::MolDesc) * nmol;
    const size_t c_off = (dbytes + 255) & ~(size_t)255;
    cudaError_t e = cudaMalloc(&b->block, c_off + 256);
    if (e == cudaSuccess) e = cudaMemcpy(b->block, descs.data(), dbytes, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset((char*)b->block + c_off, 0, 256);
    if (e != cudaSuccess) {
        if (b->block) cudaFree(b->block);
        free(b);
        return cuda_status(e, "okg_batch_create: device descriptors");
    }
    b->nmol = nmol;
    b->d_descs = (mx::MolDesc*)b->block;
    b->d_counter = (unsigned long long*)((char*)b->block + c_off);
    b->d_status = (int*)((char*)b->block + c_off + 64);
    b->total_tiles = tile0;
    b->sm_count = sms > 0 ? sms : 1;
    b->grab = 1;
    b->ctas = b->sm_count;
    b->smem = mx::SMEM_BYTES;
    b->layout = mx::LAYOUT_DEFAULT;
    b->cusp = any_cusp;
    e = mx::configure_kernels();
    if (e != cudaSuccess) {
        cudaFree(b->block);
        free(b);
        return cuda_status(e, "okg_batch_create: shared memory attribute");
    }
    *out = b;
    return OKG_OK;
}

extern "C" int okg_batch_destroy(okg_batch* b)
{
    if (!b) return OKG_OK;
    cudaError_t e = cudaFree(b->block);
    free(b);
    return cuda_status(e, "okg_batch_destroy");
}

extern "C" int okg_batch_set_schedule(okg_batch* b, int grab, int ctas, int threads)
{
    if (!b || grab < 1 || ctas < 1) return set_error(OKG_ERR_ARG, "okg_batch_set_schedule: grab and ctas >= 1");
    if (ctas > b->sm_count) return set_error(OKG_ERR_UNSUPPORTED, "okg_batch_set_schedule: one CTA per SM at most");
    if (threads != 256 && threads != 384 && threads != 512)
        return set_error(OKG_ERR_ARG, "okg_batch_set_schedule: threads must be 256, 384 or 512");
    b->grab = grab;
    b->ctas = ctas;
    b->layout = mx::layout_index(threads, 1);
    return OKG_OK;
}

extern "C" int okg_batch_set_generation(okg_batch* b, int threads, int points_per_thread)
{
    const int l = mx::layout_index(threads, points_per_thread);
    if (!b || l < 0)
        return set_error(OKG_ERR_ARG, "okg_batch_set_generation: (threads, points) must be (256|384|512, 1) or "
                                      "(256|384, 2)");
    b->layout = l;
    return OKG_OK;
}

extern "C" int okg_batch_tiles(const okg_batch* b, long long* total_tiles)
{
    if (!b || !total_tiles) return set_error(OKG_ERR_ARG, "okg_batch_tiles: NULL argument");
    *total_tiles = b->total_tiles;
    return OKG_OK;
}

extern "C" int okg_batch_run(okg_batch* b, okg_stream stream)
{
    if (!b) return set_error(OKG_ERR_ARG, "okg_batch_run: NULL batch");
    if (b->total_tiles == 0) return OKG_OK;
    cudaStream_t st = (cudaStream_t)stream;
    cudaError_t e = cudaMemsetAsync(b->d_counter, 0, sizeof(unsigned long long), st);
    if (e != cudaSuccess) return cuda_status(e, "okg_batch_run: counter reset");
    mx::BatchParams P;
    P.descs = b->d_descs;
    P.nmol = b->nmol;
    P.grab = b->grab;
    P.total_tiles = b->total_tiles;
    P.counter = b->d_counter;
    P.status = b->d_status;
    P.wait_limit = mx::WAIT_LIMIT;
    if (b->cusp && !mx::layout_has_cusp(b->layout))
        return set_error(OKG_ERR_UNSUPPORTED, "okg_batch_run: the FP64 cusp points need one point per generation thread");
    const long long grid = b->total_tiles < b->ctas ? b->total_tiles : b->ctas;
    mx::launch_batch(b->layout, b->cusp, (unsigned)grid, st, P);
    return cuda_status(cudaGetLastError(), "okg_batch_run launch");
}

extern "C" int okg_batch_status(okg_batch* b, int* device_status)
{
    if (!b || !device_status) return set_error(OKG_ERR_ARG, "okg_batch_status: NULL argument");
    int v = 0;
    cudaError_t e = cudaMemcpy(&v, b->d_status, sizeof(int), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_status(e, "okg_batch_status");
    *device_status = v;
    if (v) {
        cudaMemset(b->d_status, 0, sizeof(int));
        if (v & 1) return set_error(OKG_ERR_TIMEOUT, "okg_batch_run: a tensor-core wait timed out");
        return set_error(OKG_ERR_UNSUPPORTED, "okg_batch_run: more than 8 cusp atoms in one 128-point tile");
    }
    return OKG_OK;
}

extern "C" int okg_mixed_status(okg_mixed_plan* p, int* device_status)
{
    if (!p || !device_status) return set_error(OKG_ERR_ARG, "okg_mixed_status: NULL argument");
    int v = 0;
    cudaError_t e = cudaMemcpy(&v, p->status, sizeof(int), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_status(e, "okg_mixed_status");
    *device_status = v;
    if (v) {
        cudaMemset(p->status, 0, sizeof(int));
        if (v & 1) return set_error(OKG_ERR_TIMEOUT, "okg_rho_mixed: a tensor-core wait timed out");
        return set_error(OKG_ERR_UNSUPPORTED, "okg_rho_mixed: more than 8 cusp atoms in one 128-point tile");
    }
    return OKG_OK;
}

// ---------------------------------------------------------------------------
// Allocation-free variant of okg_rho_mixed.
//
// Some callers cannot allocate device memory at the point where they evaluate the
// density: code that runs inside a framework which owns all device memory through
// its own pool, or a real-time loop that cannot pay the implicit device-wide
// synchronisation of cudaMalloc/cudaFree.  They still need the tensor-core path
// with fresh MO coefficients on every call, which normally goes through a plan
// (okg_mixed_plan_create allocates the split-coefficient buffer).  This entry
// point instead uses one file-scope device array as its scratch: the BF16 operand
// tiles of the coefficients, the padded occupations and the timeout status word.
//
// * Limit: OKG_NOALLOC_SCRATCH_BYTES (2 MiB) of scratch per device; larger
//   (basis, nmo) combinations are rejected with OKG_ERR_UNSUPPORTED.  Every GPU
//   that loads the library holds the array until the process exits.
// * The first call on a device looks up the array's device address
//   (cudaGetSymbolAddress) and sets the kernel's shared-memory attribute, with that
//   device current; make that first call before any stream capture.  The address
//   is kept for the life of the process: do not use the entry point across a
//   cudaDeviceReset (which invalidates it).
// * The caller passes a device int for the timeout status (required): the call
//   clears it on the stream and the kernel sets it to 1 if a tensor-core wait
//   expired, in which case the outputs are incomplete.
// * All calls on a device share the one array and it keeps the last call's
//   contents: calls that overlap on the GPU (different streams, or host threads
//   that do not order their streams) race on it.  Each call rewrites every byte it
//   reads and clears the tile counter before its kernels run.
// * Like okg_rho_mixed, it evaluates every point on the tensor cores: the points
//   near nuclei are not recomputed in FP64 (the Python layer does that for the
//   plan path).
// ---------------------------------------------------------------------------
#include <mutex>

namespace okg {
namespace mx {
constexpr size_t NOALLOC_SCRATCH_BYTES = 2u << 20;
static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_SCRATCH_BYTES];

struct NoallocDevice {
    unsigned char* base = nullptr;  // device address of g_noalloc_scratch on this device
    int sm_count = 0;
    bool ready = false;
};
static NoallocDevice g_noalloc_dev[64];
static std::mutex g_noalloc_mu;

}  // namespace mx
}  // namespace okg

extern "C" int okg_rho_mixed_noalloc(const okg_basis* b, const okg_grid* gr, int nmo, const double* d_coeff,
                                     const double* d_occ, int want_grad, double* d_rho, double* d_grad, int64_t ld,
                                     int* d_status, okg_stream stream)
{
    using namespace okg::mx;
    if (!b || !gr || !d_coeff || !d_occ || !d_rho || (want_grad && !d_grad) || nmo <= 0)
        return set_error(OKG_ERR_ARG, "okg_rho_mixed_noalloc: NULL argument or nmo <= 0");
    // the timeout status goes to the caller's word: a word inside the shared scratch
    // could not be read back, and an expired wait would go unnoticed
    if (!d_status) return set_error(OKG_ERR_ARG, "okg_rho_mixed_noalloc: d_status is NULL");
    Grid g;
    g.x = gr->d_x;
    g.y = gr->d_y;
    g.z = gr->d_z;
    g.npts = gr->npts;
    g.offset = gr->offset;
    g.nx = gr->nx;
    g.ny = gr->ny;
    g.nz = gr->nz;
    g.regular = gr->regular;
    if (g.npts < 0 || !g.x || !g.y || !g.z) return set_error(OKG_ERR_ARG, "okg_rho_mixed_noalloc: bad grid");
    if (g.regular && (g.nx <= 0 || g.ny <= 0 || g.nz <= 0 || g.offset < 0 ||
                      g.offset + g.npts > (long long)g.nx * g.ny * g.nz))
        return set_error(OKG_ERR_ARG, "okg_rho_mixed_noalloc: regular grid range outside Nx*Ny*Nz");
    if (ld < g.npts) return set_error(OKG_ERR_ARG, "okg_rho_mixed_noalloc: ld < npts");

    // scratch layout: split coefficients | occupations | tile counter
    const int npass = (nmo + NMAX - 1) / NMAX;
    const int per = (nmo + npass - 1) / npass;
    const int npad = (per + 15) / 16 * 16;
    const size_t bpack_bytes = (size_t)npass * b->dev.nmchunk * 3 * npad * ROWB;
    const size_t occ_off = (bpack_bytes + 255) & ~(size_t)255;
    const size_t st_off = occ_off + (((size_t)4 * npass * npad * 8 + 255) & ~(size_t)255);
    if (b->dev.nshell > MAX_SHELLS || b->dev.nmchunk > MAX_CHUNKS)
        return set_error(OKG_ERR_UNSUPPORTED, "okg_rho_mixed_noalloc: more than 2048 shells or 192 column chunks");
    if (b->dev.max_nprim > MAX_PRIM)
        return set_error(OKG_ERR_UNSUPPORTED, "okg_rho_mixed_noalloc: a shell with more than 31 primitives");
    if (st_off + 256 > NOALLOC_SCRATCH_BYTES)
        return set_error(OKG_ERR_UNSUPPORTED,
                         "okg_rho_mixed_noalloc: this basis and MO count need more than the 2 MiB of static "
                         "scratch; use okg_mixed_plan_create / okg_rho_mixed");
    b->mixed_locked = 1;  // the column order read by the launch below stays as it is

    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_status(e, "okg_rho_mixed_noalloc: cudaGetDevice");
    if (dev < 0 || dev >= 64) return set_error(OKG_ERR_DEVICE, "okg_rho_mixed_noalloc: device index above 63");
    NoallocDevice* nd = &g_noalloc_dev[dev];
    {
        std::lock_guard<std::mutex> lock(g_noalloc_mu);
        if (!nd->ready) {
            int major = 0, minor = 0, sms = 0;
            cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev);
            cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev);
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
            if (major != 10 || minor != 3) return set_error(OKG_ERR_DEVICE, "okg_rho_mixed_noalloc: needs an sm_103 GPU");
            void* ptr = nullptr;
            e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
            if (e != cudaSuccess) return cuda_status(e, "okg_rho_mixed_noalloc: cudaGetSymbolAddress");
            e = configure_kernels();
            if (e != cudaSuccess) return cuda_status(e, "okg_rho_mixed_noalloc: shared memory attribute");
            nd->base = (unsigned char*)ptr;
            nd->sm_count = sms;
            nd->ready = true;
        }
    }
    if (g.npts == 0) return OKG_OK;
    cudaStream_t st = (cudaStream_t)stream;
    __nv_bfloat16* bpack = (__nv_bfloat16*)nd->base;
    double* occ = (double*)(nd->base + occ_off);
    int* status = d_status;
    e = cudaMemsetAsync(status, 0, sizeof(int), st);
    if (e != cudaSuccess) return cuda_status(e, "okg_rho_mixed_noalloc: clear status");
    const BasisDev& B = b->dev;
    pack_b_kernel<<<nd->sm_count * 4, 256, 0, st>>>(d_coeff, nmo, B.ncart, B.mcol_cart, B.mcol_g, B.nmchunk, npass, npad,
                                                    bpack);
    pack_occ_kernel<<<(npass * npad + 127) / 128, 128, 0, st>>>(d_occ, nmo, npass * npad, occ);
    Params P;
    make_desc(P.D, B, g, bpack, occ, npass, npad, nmo, want_grad, d_rho, d_grad, ld);
    P.status = status;
    P.counter = (unsigned long long*)(nd->base + st_off + 64);
    P.wait_limit = WAIT_LIMIT;
    e = cudaMemsetAsync(P.counter, 0, sizeof(unsigned long long), st);
    if (e != cudaSuccess) return cuda_status(e, "okg_rho_mixed_noalloc: counter reset");
    const long long grid = P.D.ntiles < nd->sm_count ? P.D.ntiles : nd->sm_count;
    launch_single(LAYOUT_DEFAULT, false, (unsigned)grid, st, P);
    return cuda_status(cudaGetLastError(), "okg_rho_mixed_noalloc launch");
}
