// Tensor-core (tcgen05, sm_103a) building blocks and the emulated-FP64 layout
// of the per-mode inverses.
//
// Emulated FP64 products (an Ozaki-style split into exact integer slices):
// a matrix row is scaled by a power of two 2^e with |a_ij| < 2^e, rounded to
// the integer U = round(a 2^(54-e)) (|U| <= 2^54) and written in 8 balanced
// base-128 digits, U = sum_s c_s 128^(7-s), c_s in [-64, 63]; a right-hand
// side column likewise with its own power of two 2^f.  Every digit is an
// integer that FP16 holds exactly, so one tcgen05.mma (kind::f16, FP32
// accumulation) of two digit matrices is exact while its sums stay below 2^24:
// |c d| <= 2^12, times at most 128 terms of K, times at most 8 digit pairs
// summed into one accumulator, is at most 2^22.  The 36 pairs (s, t) with
// s + t <= 7 go into 8 accumulators by weight class c = s + t, combined in
// 64-bit integers as T = sum_{c<=6} D_c 128^(6-c) + round(D_7 / 128)
// (|T| < 2^62), and a b = T 2^(e+f-52) up to the dropped classes and that
// rounding: an error of about 2^-53 of the product of the row and column
// scales, one int64->FP64 conversion and one power-of-two scaling per output
// instead of a K-term FP64 dot product.
//
// Operators are folded into even and odd blocks (centro-symmetric: diag(Ge,
// Go); centro-antisymmetric: [[0, De], [Do, 0]]).  Each block is its own
// M = 128 MMA on its own rows: block E (the even output rows, e8 of them) and
// block O (the odd output rows, o8), so a block of up to 128 rows fits, i.e.
// nz <= 255.  The right-hand sides hold the even input levels at K indices
// [0, ke) and the odd ones at [ke, ke + ko) (each padded to a multiple of 16
// for the MMA K-steps); a symmetric block E reads K [0, ke) and block O reads
// [ke, ke + ko); an antisymmetric block E (De) reads the odd inputs and block
// O (Do) the even ones.  Rows past a block's e8 or o8 are whatever follows in
// shared memory: the MMA reads them, and their products land in TMEM lanes
// that are never read.
//
// Shared-memory operands: K-major, no swizzle, "core matrices" of 8 rows x 8
// FP16 (16 bytes per row, 128 bytes per core matrix); K-adjacent core
// matrices are 128 B apart (LBO), 8-row groups (K width x 2) B apart (SBO).
#pragma once

#include <cuda_fp16.h>
#include <cstdint>

namespace dns3d {

constexpr int kTcSlices = 8;    // digits per value
constexpr int kTcClasses = 8;   // digit-pair weight classes kept (s + t <= 7)
constexpr int kTcFixBits = 54;  // U = round(a 2^(54-e))
constexpr int kTcN = 16;        // MMA N: columns of one right-hand-side block
constexpr int kTcM = 128;       // MMA M (rows beyond a block's size are ignored)
constexpr int kTcDCols = kTcClasses * kTcN;  // TMEM columns of one block's accumulators

// Folded operator geometry: even block he x he (symmetric) or he x ho
// (antisymmetric), odd block ho x ho or ho x he; rows padded to multiples of
// 8 (e8, o8; m8 = e8 + o8 rows of row exponents, even rows first), K widths
// padded to multiples of 16 (ke, ko; kt = ke + ko right-hand-side rows).
struct TcGeom {
    int he, ho, e8, o8, m8, ke, ko, kt, ncore_e, ncore_o;
};

__host__ __device__ inline TcGeom tc_geom(int nz) {
    TcGeom t;
    t.ho = nz / 2;
    t.he = nz - t.ho;
    t.e8 = (t.he + 7) / 8 * 8;
    t.o8 = (t.ho + 7) / 8 * 8;
    t.m8 = t.e8 + t.o8;
    t.ke = (t.he + 15) / 16 * 16;
    t.ko = (t.ho + 15) / 16 * 16;
    t.kt = t.ke + t.ko;
    t.ncore_e = (t.e8 / 8) * (t.e8 / 8);
    t.ncore_o = (t.o8 / 8) * (t.o8 / 8);
    return t;
}

// Each folded block must fit one M = 128 MMA (and the K of one MMA, 128, in
// the exactness bound above).
__host__ __device__ inline bool tc_supported(int nz) { return tc_geom(nz).ke <= kTcM; }

// K widths of blocks E and O and the K offsets of their right-hand-side rows:
// symmetric E = Ge (ke, inputs at 0), O = Go (ko, inputs at ke); antisymmetric
// E = De (ko, the odd inputs at ke), O = Do (ke, the even inputs at 0).
struct TcBlocks {
    int kE, kO, bE, bO;
    int aE, a;  // halves of block E, of one digit slice (E then O)
};

__host__ __device__ inline TcBlocks tc_blocks(const TcGeom& t, bool anti) {
    TcBlocks b;
    b.kE = anti ? t.ko : t.ke;
    b.kO = anti ? t.ke : t.ko;
    b.bE = anti ? t.ke : 0;
    b.bO = anti ? 0 : t.ke;
    b.aE = t.e8 * b.kE;
    b.a = b.aE + t.o8 * b.kO;
    return b;
}

// Row of the folded value (even rows first, odd ones from e8) behind
// right-hand-side K index kk, or -1 for a padding K row.
__host__ __device__ inline int tc_k_row(const TcGeom& t, int kk) {
    return kk < t.ke ? (kk < t.he ? kk : -1) : (kk - t.ke < t.ho ? t.e8 + (kk - t.ke) : -1);
}

// Entries per q of the fixed-point Poisson inverses (folded blocks he x he
// and ho x ho), padded to an even count so that every q's block starts on a
// 16-byte boundary (the solve stages them with 16-byte copies).
__host__ __device__ inline size_t fx_qstride(int he, int ho) {
    return ((size_t)he * he + (size_t)ho * ho + 1) / 2 * 2;
}

// Halves per q of the compact slice store: per digit, the nonzero core
// matrices (even block row-major, then odd block), 64 halves each.
__host__ __device__ inline size_t tc_q_halves(const TcGeom& t) {
    return (size_t)kTcSlices * (t.ncore_e + t.ncore_o) * 64;
}

// Offset (in halves) of element (r, k) of a K-major operand of K width kw.
__host__ __device__ inline int tc_core_off(int r, int k, int kw) {
    return ((r >> 3) * (kw >> 3) + (k >> 3)) * 64 + (r & 7) * 8 + (k & 7);
}

// Balanced base-128 digits of |U| <= 2^54, most significant first.
__device__ __forceinline__ void tc_digits(long long u, int* c) {
#pragma unroll
    for (int s = kTcSlices - 1; s >= 0; --s) {
        const int r = (int)(u & 127);
        const int d = r >= 64 ? r - 128 : r;
        c[s] = d;
        u = (u - d) >> 7;
    }
}

// 64 in each of the 8 base-128 digit places: 64 (1 + 128 + ... + 128^7).
constexpr unsigned long long kTcDigitBias = 0x0081020408102040ULL;

__device__ __forceinline__ __half2 tc_u32_as_half2(uint32_t w) {
    __half2 h;
    memcpy(&h, &w, sizeof(h));
    return h;
}

// The digits of two values at once (K rows kk, kk + 1 of one right-hand-side
// column), slice s as the pair {c_s(u0), c_s(u1)}: the same digits as
// tc_digits.  V = U + kTcDigitBias holds U's balanced digits plus 64 in its
// 7-bit fields (0 <= V < 2^56 for |U| <= 2^54, no carries), and for a field
// value v in [0, 127] the FP16 with bits 0x6400 | v is 1024 + v, so one
// packed subtraction of 1088 gives a pair of digits.
__device__ __forceinline__ void tc_digit_pairs(long long u0, long long u1, __half2* h) {
    const unsigned long long v0 = (unsigned long long)u0 + kTcDigitBias;
    const unsigned long long v1 = (unsigned long long)u1 + kTcDigitBias;
    const uint32_t l0 = (uint32_t)v0, m0 = (uint32_t)(v0 >> 28);
    const uint32_t l1 = (uint32_t)v1, m1 = (uint32_t)(v1 >> 28);
    const __half2 off = tc_u32_as_half2(0x64406440u);  // {1088, 1088}
#pragma unroll
    for (int fi = 0; fi < kTcSlices; ++fi) {  // fi = 0: least significant digit (slice 7)
        const uint32_t a = fi < 4 ? l0 >> (7 * fi) : m0 >> (7 * (fi - 4));
        const uint32_t b = fi < 4 ? l1 >> (7 * fi) : m1 >> (7 * (fi - 4));
        const uint32_t w = __byte_perm((a & 127u) | 0x6400u, (b & 127u) | 0x6400u, 0x5410);
        h[kTcSlices - 1 - fi] = __hsub2(tc_u32_as_half2(w), off);
    }
}

// round(x 2^(B-f)) for |x| < 2^f (|result| <= 2^B), from the bits of x
// (integer operations only).
template <int B>
__device__ __forceinline__ long long tc_fixed_bits(double x, int f) {
    const long long b = __double_as_longlong(x);
    int ex = (int)((b >> 52) & 0x7FF);
    long long m = b & 0xFFFFFFFFFFFFFLL;
    if (ex == 0) {
        if (m == 0) return 0;
        ex = 1;  // subnormal: no implicit bit
    } else {
        m |= 1LL << 52;
    }
    const int sh = 1075 - B + f - ex;  // x = m 2^(ex-1075); U = m 2^(ex-1075+B-f)
    if (sh >= 62) return 0;
    const long long u = sh > 0 ? (m + (1LL << (sh - 1))) >> sh : m << (-sh);
    return b < 0 ? -u : u;
}

// round(x 2^(54-f)) for |x| < 2^f: the digit scheme's fixed point.
__device__ __forceinline__ long long tc_fixed(double x, int f) { return tc_fixed_bits<kTcFixBits>(x, f); }

// Smallest f with |x| < 2^f for the largest |x| given by its bits (0 if zero).
__device__ __forceinline__ int tc_exponent(unsigned long long absbits) {
    if (absbits == 0) return 0;
    const int ex = (int)(absbits >> 52);
    return (ex == 0 ? -1022 : ex - 1023) + 1;
}

// A 32-bit key of |x| that orders like |x| (the high word of |x| with the
// low word's nonzero-ness in its lowest bit), so that the largest key of a
// column gives tc_exponent of its largest |x|: tc_exponent_key below.
__device__ __forceinline__ unsigned tc_key(double x) {
    const unsigned long long ab = (unsigned long long)__double_as_longlong(x) & 0x7FFFFFFFFFFFFFFFULL;
    return (unsigned)(ab >> 32) | ((unsigned)ab != 0u ? 1u : 0u);
}
__device__ __forceinline__ int tc_exponent_key(unsigned key) {
    if (key == 0) return 0;
    const int ex = (int)(key >> 20);
    return (ex == 0 ? -1022 : ex - 1023) + 1;
}

// Exact FP32 integer (|v| < 2^22) to int.
__device__ __forceinline__ int tc_f2i(float v) { return __float_as_int(v + 12582912.0f) - 0x4B400000; }

// The whole combination T of one output from its 8 class accumulators (as
// raw TMEM words), T = sum_{c<=6} D_c 128^(6-c) + round(D_7 / 128) with
// D_c = tc_f2i of class c (see the header comment): adjacent
// classes pair up exactly in 32 bits (|D_c 128 + D_c+1| < 2^30), so only
// three 64-bit steps remain.
__device__ __forceinline__ long long tc_combine8(uint32_t w0, uint32_t w1, uint32_t w2, uint32_t w3, uint32_t w4,
                                                 uint32_t w5, uint32_t w6, uint32_t w7) {
    const int pa = tc_f2i(__uint_as_float(w0)) * 128 + tc_f2i(__uint_as_float(w1));
    const int pb = tc_f2i(__uint_as_float(w2)) * 128 + tc_f2i(__uint_as_float(w3));
    const int pc = tc_f2i(__uint_as_float(w4)) * 128 + tc_f2i(__uint_as_float(w5));
    const int tail = tc_f2i(__uint_as_float(w6)) + ((tc_f2i(__uint_as_float(w7)) + 64) >> 7);
    long long T = (long long)pa * 16384 + pb;
    T = T * 16384 + pc;
    return T * 128 + tail;
}

__device__ __forceinline__ uint32_t tc_smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ uint64_t tc_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFF);
    d |= (uint64_t)((lbo >> 4) & 0x3FFF) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFF) << 32;
    d |= (uint64_t)1 << 46;  // descriptor version of the sm_100 family; no swizzle, base offset 0
    return d;
}

// kind::f16 instruction descriptor: FP32 accumulator, FP16 A and B, both
// K-major, M = kTcM, N = n (a multiple of 16 up to 256).
__device__ __forceinline__ uint32_t tc_idesc(int n) {
    return (1u << 4) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(kTcM >> 4) << 24);
}

__device__ __forceinline__ void tc_alloc(uint32_t* dst_smem, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(tc_smem_u32(dst_smem)),
                 "r"(ncols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
}

__device__ __forceinline__ void tc_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols));
}

__device__ __forceinline__ void tc_mma(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d_tmem),
        "l"(a), "l"(b), "r"(idesc), "r"(acc));
}

// Arms the barrier's current phase for `bytes` of asynchronous copies (one arrival).
__device__ __forceinline__ void tc_mbar_expect(uint64_t* mbar, uint32_t bytes) {
    asm volatile(
        "{\n\t.reg .b64 st;\n\t"
        "mbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n\t}\n" ::"r"(tc_smem_u32(mbar)),
        "r"(bytes));
}

// Bulk copy global -> shared (16-byte aligned, size a multiple of 16),
// completing on the barrier's transaction count.
__device__ __forceinline__ void tc_bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* mbar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            tc_smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(tc_smem_u32(mbar))
        : "memory");
}

// Asynchronous 16-byte global -> shared copy (L2 only), its commit and the
// wait for all of this thread's outstanding groups.
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(tc_smem_u32(smem)), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }
// ... all but the most recent group
__device__ __forceinline__ void cp_async_wait_one() { asm volatile("cp.async.wait_group 1;" ::: "memory"); }

__device__ __forceinline__ void tc_commit(uint64_t* mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
        tc_smem_u32(mbar)));
}

__device__ __forceinline__ void tc_mbar_init(uint64_t* mbar, uint32_t count = 1) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(tc_smem_u32(mbar)), "r"(count));
    asm volatile("fence.mbarrier_init.release.cluster;");
}

// Waits for phase `parity` of the barrier, at most `limit` polls; true if it completed.
__device__ __forceinline__ bool tc_mbar_wait(uint64_t* mbar, uint32_t parity, int limit) {
    uint32_t done = 0;
    for (int it = 0; it < limit && !done; ++it) {
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}\n"
            : "=r"(done)
            : "r"(tc_smem_u32(mbar)), "r"(parity));
    }
    return done != 0;
}

// TMEM loads issued back to back with one wait (tc_ld_wait) for all of them:
// N = 2 or 4 consecutive columns of this thread's lane, no wait.
__device__ __forceinline__ void tc_ld2_nw(uint32_t taddr, uint32_t* r) {
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x2.b32 {%0,%1}, [%2];" : "=r"(r[0]), "=r"(r[1]) : "r"(taddr));
}
__device__ __forceinline__ void tc_ld4_nw(uint32_t taddr, uint32_t* r) {
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0,%1,%2,%3}, [%4];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(taddr));
}
// The wait, then every loaded register passed through an empty volatile asm
// ordered after it, so that no use of a loaded value moves above the wait.
template <int N>
__device__ __forceinline__ void tc_ld_wait(uint32_t (&r)[N]) {
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < N; ++i) asm volatile("" : "+r"(r[i]));
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;"); }
// generic-proxy shared-memory writes visible to the tensor cores
__device__ __forceinline__ void tc_fence_proxy() { asm volatile("fence.proxy.async.shared::cta;"); }

}  // namespace dns3d
