// sfb_split.cu -- split-precision raw SFB on the tcgen05 tensor cores (sm_103a).
//
// f_l(m, n) = k_ln * sum_i w_i j_l(k_ln r_i) P_lm(x_i) e^{-i m phi_i}  (sfb_raw.cpp:56-84)
// computed per multipole l as the product D[n][col] = sum_i J[n][i] Y[i][col] with
//   J[n][i] = w_i j_l(k_ln r_i) * 2^sJ          (A operand, 128 x K, FP16 hi + lo)
//   Y[i][2m+0/1] = Re/Im P_lm(x_i) e^{-im phi_i} * 2^12   (B operand, K x 2 mcount)
// and three tcgen05.mma kind::f16 products per K = 16 step (Jhi*Yhi + Jhi*Ylo +
// Jlo*Yhi).  Both operands are scaled by powers of two towards the top of the FP16
// range so the lo halves stay normal.
//
// Work split: one launch per l; a CTA owns one work item: a catalog, a block of <= 128
// complex m (so l >= 128 uses two items per slab, each generating the J tile), a half
// of <= 128 radial orders (nmax > 128 uses two, each generating the Y tile; the first
// writes the Legendre rows) and a slab of 32-point tiles.
// Accumulation: the tensor core accumulates one tile (6 MMAs) into D_tile in tensor
// memory; the CTA then folds D_tile into a second tensor-memory region D_acc with
// FP32 round-to-nearest adds on the CUDA cores (the tensor core's own FP32
// accumulation drifts measurably over long chains), and every FLUSH_FOLDS tiles adds
// D_acc into the CTA's FP32 partial in global memory.  k_split_reduce sums the slab
// partials in FP64 in fixed order and applies k_ln.
//
// Operand generation (CUDA cores, FP32 with float-float inputs):
//   * j_l from a per-l piecewise degree-6 polynomial on unit intervals of z = k r
//     centred on the integers (Chebyshev interpolation of the FP64 j_l, monomial
//     coefficients in u = z - round(z) in [-1/2, 1/2]; error <= ~1e-7 of the envelope,
//     dominated by the FP32 coefficients), the argument formed as a float-float
//     product so its absolute error is ~1e-12;
//   * P_lm by one step of the l-recurrence from FP32 rows P_{l-1}, P_{l-2} in HBM
//     (staged into shared memory one tile ahead by TMA), with the recurrence
//     coefficients and x = cos(theta), s = sin(theta) as float-float pairs; the rows
//     are stored scaled by 2^100 so that sectoral seeds down to 2^-226 stay
//     representable (enough for lmax <= 256; above, each value carries a 2-bit exponent);
//     the m = 0 step is rounded once (step_once), so Y_l0 carries no mean error over the
//     sphere through which a catalog's monopole could leak into l > 0.  With
//     CATANA_SPLIT_ACCURATE, and always above lmax 256, the columns m < 128 follow the
//     Reinsch-modified recurrence at |cos(theta)| instead (rows P_l and
//     D_l = P_l - rho_l P_{l-1}), whose rounding does not build up near the poles;
//   * the sectoral seeds stay FP64: before the level loop, k_split_sectoral advances
//     every point's P_ll = -sqrt((2l+1)/(2l)) s P_{l-1,l-1} in FP64 from the FP32
//     value of P_00 and stores each level's P_ll, rounded once, in slot m = l of the
//     P_{l-1} row set -- a slot no level uses before level l reads it, and one the
//     TMA staging of P_{l-1} already covers -- so column m of the FP32 recurrence
//     starts from a correctly rounded P_mm instead of m rounded FP32 steps;
//   * e^{-i m phi}: one sincospif of the exact phase (64-bit fixed-point fraction of a
//     turn) per warp-run of <= 8 m, then complex rotation by e^{i phi}.
// Pipeline: two operand buffers and two row stages.  Warps 0..15 generate the operands
// of tile t+1 while the tensor core multiplies tile t; warps 16..19 (one per TMEM lane
// quadrant) fold D_tile into D_acc, flush, and issue each tile's MMAs, so the fold no
// longer sits between a CTA barrier and the next MMA.  Hand-offs are mbarriers: operands
// written, MMAs complete, row stage read.  Every wait is bounded (1 s); on timeout the
// kernel records CATANA_ERR_CUDA in the error word, stops issuing work and frees its
// tensor memory.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "common.cuh"
#include "special.cuh"
#include "tc05.cuh"

namespace catana_gpu {

namespace {

constexpr int KT = 32;              // points per tile (two K=16 MMA steps)
constexpr int NOPW = 16;            // operand warps
constexpr int NTHR = 32 * NOPW;
constexpr int QPW = (32 + NOPW - 1) / NOPW;   // most quads of complex m per operand warp (128 m = 32 quads)
constexpr int JPW = (64 + NOPW - 1) / NOPW;   // most J row pairs per operand warp (128 rows)
static_assert(JPW <= 16, "k_split_l: one lane per J row in the Taylor coefficients");
constexpr int NFOLDW = 4;           // fold / MMA warps, one per TMEM lane quadrant
constexpr int NTOT = NTHR + 32 * NFOLDW;
constexpr int MBLK = 128;           // complex m per CTA block (256 accumulator columns)
constexpr int FOLD_TILES = 1;       // tiles accumulated by the tensor core before a fold into D_acc (2 doubles the C_l error)
constexpr int FLUSH_FOLDS = 128;    // folds into the TMEM sum before it goes to global memory
constexpr int NINT_MAX = 1664 - (NOPW * JPW - 64);  // table intervals resident in shared memory (lmax 512, nmax 256 at r <= rmax: 1522)
constexpr double H = 1.0;           // table interval width in z (intervals centred on integers)
constexpr int TDEG = 6;             // table polynomial degree (7 coefficients in two float4)
constexpr int SPLIT_LMAX = 256;     // rows scaled by 2^100 alone cover l < 256 (see header comment)
constexpr int SPLIT_LMAX_EXT = 512; // with the 2-bit row exponents (extended range)
constexpr int SPLIT_NMAX = 256;     // two 128-lane halves (separate work items)
constexpr int NHALF = 128;          // radial orders per work item (accumulator lanes)
constexpr int MR_STD = 128;         // Reinsch-modified rows: columns m >= MR_STD keep the three-term step
constexpr uint64_t WAIT_NS = 1000000000ull;  // drains of in-flight copies and MMAs before exit (1 s)

// shared-memory map (bytes, from a 1024-aligned base)
constexpr uint32_t SM_J = 8192;          // J hi or J lo: 4 k-groups x 2 atoms
constexpr uint32_t SM_Y = 16384;         // Y hi or Y lo: 4 k-groups x 4 atoms (256 columns)
constexpr uint32_t SM_BUF = 2 * SM_J + 2 * SM_Y;
constexpr uint32_t OFF_ST = 2 * SM_BUF;                // staged tiles: NST stages (2 or 3)
constexpr uint32_t SM_STROW = MBLK * KT * 4;           // one row set (MBLK m x 32 points) = 16 KB
constexpr uint32_t SM_STPTS = KT * 48;                 // the tile's 32 SplitPt records
constexpr uint32_t SM_STEXP = MBLK * 8;                // row exponent words of one row set (extended range)
// one stage: P_{l-1}, P_{l-2} (Reinsch-modified rows: X_{l-1}), the points and, extended
// range, the exponent words (one word serves P_{l-1} and X_{l-1})
__host__ __device__ constexpr uint32_t sm_stage(bool ext, bool rs) {
    return 2 * SM_STROW + SM_STPTS + (ext ? SM_STEXP : 0u);
}
// after the stages: per n pair (kz_hi, kz_lo) x 2; J scale 2^s_ln per n; readout 2^-s_ln 2^-12 per
// n; recurrence coefficients of the m pairs (and of the Reinsch-modified step); per operand warp
// the Taylor coefficients of its 8 J rows; last, the j_l table of the launch (its interval count
// sets the dynamic size)
__host__ __device__ constexpr uint32_t off_kz(bool ext, bool rs, int nst) {
    return OFF_ST + (uint32_t)nst * sm_stage(ext, rs);
}
__host__ __device__ constexpr uint32_t off_js(bool ext, bool rs, int nst) { return off_kz(ext, rs, nst) + NHALF * 8; }
__host__ __device__ constexpr uint32_t off_inv(bool ext, bool rs, int nst) { return off_js(ext, rs, nst) + NHALF * 4; }
__host__ __device__ constexpr uint32_t off_coef(bool ext, bool rs, int nst) { return off_inv(ext, rs, nst) + NHALF * 4; }
__host__ __device__ constexpr uint32_t off_rcoef(bool ext, bool rs, int nst) { return off_coef(ext, rs, nst) + MBLK * 16; }
__host__ __device__ constexpr uint32_t off_jt(bool ext, bool rs, int nst) { return off_rcoef(ext, rs, nst) + MBLK * 16; }
__host__ __device__ constexpr uint32_t off_tab(bool ext, bool rs, int nst) {
    return off_jt(ext, rs, nst) + (uint32_t)NOPW * JPW * 8 * 4;
}
// dynamic shared memory of a launch (+ 1024 B of alignment slack)
constexpr uint32_t smem_bytes(bool ext, bool rs, int nst, int nint) {
    return off_tab(ext, rs, nst) + (uint32_t)nint * 32 + 1024;
}
constexpr uint32_t SMEM_LIMIT = 232448 - 1024;  // per block, leaving room for the static part
static_assert(smem_bytes(true, true, 2, NINT_MAX) <= SMEM_LIMIT, "k_split_l shared memory");
// J of a tile comes from a cubic Taylor expansion about its record-16 radius when
// k_max max|r - r_c| <= JT_TAU: the omitted terms are below JT_TAU^4 / 24 ~ 7e-9 of j_l's
// envelope (the interpolant's derivatives are bounded by it)
constexpr float JT_TAU = 0.02f;

constexpr float P00_SCALED = 0.28209479177387814347f * 1.2676506002282294e30f;  // 1/sqrt(4 pi) * 2^100
// Y operand = P * 2^12: the stored rows carry 2^100, so the readout factor is 2^-88.
// Scaling both operands towards the top of the FP16 range keeps the lo halves normal.
constexpr float Y_UNSCALE = 3.2311742677852644e-27f;  // 2^-88
constexpr float Y_SCALE = 4096.0f;                    // 2^12

// Per-point operand inputs of the split form (48 bytes, radius-sorted order).
struct SplitPt {
    float r_hi, r_lo, w;        // radius (float-float), weight
    float x_hi, x_lo;           // cos(theta); Reinsch-modified rows: |cos(theta)| (float-float)
    float s_hi, s_lo;           // sin(theta); Reinsch-modified rows: 1 - |cos(theta)| (float-float)
    float cphi, sphi;           // e^{i phi}
    float dr;                   // r - r of the tile's record 16; record 16 itself: max |dr| of the tile
    unsigned long long u;       // phi / 2pi as a 64-bit fraction of a turn
};
static_assert(sizeof(SplitPt) == 48, "SplitPt layout");

// One catalog (or catalog chunk) of a split-form plan.
struct SplitCat {
    const SplitPt *pts;     // radius-sorted point records, padded to whole tiles
    float *rows;            // Legendre row sets with m pairs interleaved per point: value (m, i) of set k
                            // at rows + k * stride * lrp + 2 stride (m / 2) + 2 i + m % 2.
                            // Reinsch-modified rows: sets 0, 1 = P_l by the parity of l, sets 2, 3 =
                            // X_l likewise; three-term rows: sets l % 3 = P_l
    int64_t n;              // points
    int stride;             // row stride (multiple of 32, >= n)
    int lrows;              // rows per set (the catalog's lmax)
    int lrp;                // lrows rounded up to even (m pairs per tile block: lrp / 2)
    int kzw;                // row width of kz (the catalog's nmax)
    int epitch;             // exponent words per tile (lrows rounded up to even)
    unsigned long long *rexp;  // extended range: exponent sets [tile][lrows] by the parity of l, set k at
                               // rexp + k * eset (one word per value serves P_l and X_l)
    int64_t eset;           // words per exponent set
    const char *tmaps;      // TMA descriptors (128 B each): rows of sets 0..3, exponent words of sets 0, 1 at 4, 5
    const float4 *kz;       // [l][kzw]: (k_ln / H as float-float, J scale 2^s_ln, 1 / (2^s_ln 2^12))
    const int *nmax_l;      // [l]: radial orders computed at l (kmax cut)
};

// One CTA of a level launch: a catalog, a block of complex m, a range of tiles.
struct SplitItem {
    int cat, mb0, mcount, n0;  // n0: first radial order of the item's 128-lane half
    int64_t t0, t1;
};

struct SplitArgs {
    int l, nint;
    const SplitItem *items;  // this level's items (one per CTA)
    const SplitCat *cats;
    const float4 *coef;      // recurrence coefficients (A, B as float-float), row l
    const float4 *rcoef;     // Reinsch-modified step (c1, rho as float-float), row l
    const float4 *tab;       // j_l table, row l: nint intervals x 2 float4
    float *partial;          // [item][256][128]
    int *err;
    uint64_t wait_ns;        // limit of every pipeline wait (1 s; a test hook shortens it)
    int stall;               // test hook: withhold the first operand hand-off of every item
};

// FP16 hi + lo halves of eight values, value pairs (columns 2k, 2k+1) from v[k], with packed
// FP32 arithmetic: hi = v rounded to FP16, lo = v - hi rounded to FP16; 16 bytes of each half.
__device__ __forceinline__ void store_split8p(uint8_t *hi_base, uint8_t *lo_base, uint32_t off, float2 v0, float2 v1,
                                              float2 v2, float2 v3) {
    const float2 v[4] = {v0, v1, v2, v3};
    uint32_t h[4], o[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        __half2 hh = __float22half2_rn(v[k]);
        const float2 hf = __half22float2(hh);
        const float2 lo = __fadd2_rn(v[k], make_float2(-hf.x, -hf.y));
        __half2 ll = __float22half2_rn(lo);
        h[k] = *reinterpret_cast<uint32_t *>(&hh);
        o[k] = *reinterpret_cast<uint32_t *>(&ll);
    }
    *reinterpret_cast<uint4 *>(hi_base + off) = make_uint4(h[0], h[1], h[2], h[3]);
    *reinterpret_cast<uint4 *>(lo_base + off) = make_uint4(o[0], o[1], o[2], o[3]);
}

// 2-bit row exponent of point q from an exponent word (bit q of each half)
__device__ __forceinline__ unsigned ebits(unsigned long long w, int q) {
    return (unsigned)((w >> q) & 1ull) | ((unsigned)((w >> (32 + q)) & 1ull) << 1);
}

// Y column order inside each 8-column group of complex m0..m0+3:
//   Re m0, Re m0+1, Im m0, Im m0+1, Re m0+2, Re m0+3, Im m0+2, Im m0+3
// (value pairs of consecutive m stay adjacent for the packed arithmetic).
__host__ __device__ __forceinline__ int col_m(int col) { return 4 * (col >> 3) + (col & 1) + 2 * ((col >> 2) & 1); }
__host__ __device__ __forceinline__ int col_ri(int col) { return (col >> 1) & 1; }

// e^{i m phi} from the 64-bit phase fraction u = phi / 2pi:  (cos, sin)(2 pi frac(m u))
__device__ __forceinline__ void phase_seed(unsigned long long u, int m, float &c, float &s) {
    const unsigned long long t = (unsigned long long)m * u;  // mod 2^64: frac(m u) exactly
    const int hi = (int)(t >> 32);                           // signed: frac in [-1/2, 1/2)
    const float a = (float)hi * 4.656612873077393e-10f;      // 2^-31 -> value of 2 frac in [-1, 1)
    sincospif(a, &s, &c);
}

// One CTA: multipole l, complex m in [128 b, 128 b + 128) of it (blockIdx.y = b),
// a slab of 32-point tiles (blockIdx.x).
// EXT (lmax > 256, always with the Reinsch-modified rows, RS): rows carry a 2-bit
// exponent per (point, m) -- the stored value is P * 2^100 * 2^(128 e); e grows by one
// when a sectoral value drops below 2^-40 and shrinks by one when a value grows past 2^40
// along l, so seeds down to ~2^-520 stay exact.  P_l and D_l of a level share the
// exponent.  Values with e > 0 are below 2^-188 and enter Y as zero.
// FULLJ: every item of the launch has 128 radial orders in its half (no kmax cut):
// with 16 operand warps each evaluates 8 J rows; otherwise the items' live row pairs
// are spread over the warps and the rest of J stays zero.
// one arrival (release, CTA scope) on an mbarrier
__device__ __forceinline__ void ws_arrive(uint64_t *mbar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(tc05::smem_u32(mbar)) : "memory");
}
// named barrier 1 of the four fold warps (128 threads); fold_vote is the same barrier
// returning the AND of every fold thread's flag, so the fold warps always agree
__device__ __forceinline__ void fold_bar() { asm volatile("barrier.sync.aligned 1, 128;" ::: "memory"); }
__device__ __forceinline__ bool fold_vote(bool v) {
    int r;
    asm volatile(
        "{\n.reg .pred p, q;\nsetp.ne.s32 p, %1, 0;\nbarrier.red.and.aligned.pred q, 1, 128, p;\nselp.s32 %0, 1, 0, q;\n}"
        : "=r"(r)
        : "r"((int)v)
        : "memory");
    return r != 0;
}

// A tt - B p2 rounded once (A = ah + al, B = bh + bl as float-float): TwoSum of the two
// large products, plus their exact remainders.  The usual fma chain rounds a partial sum
// that the large B p2 dominates, so the small A_lo tt term is absorbed -- and it has a
// nonzero mean over the sphere for m = 0, which puts a monopole component into Y_l0 that
// a catalog's monopole (a sum growing like N) leaks through into l > 0.  Explicit _rn
// operations keep the compiler from contracting or reassociating the TwoSum.
__device__ __forceinline__ float step_once(float ah, float al, float bh, float bl, float tt, float p2) {
    const float p_hi = __fmul_rn(ah, tt);
    const float p_lo = fmaf(ah, tt, -p_hi);
    const float q_hi = __fmul_rn(bh, p2);
    const float q_lo = fmaf(bl, p2, fmaf(bh, p2, -q_hi));
    const float s = __fadd_rn(p_hi, -q_hi);
    const float v = __fadd_rn(s, -p_hi);
    const float se = __fadd_rn(__fadd_rn(p_hi, -__fadd_rn(s, -v)), __fadd_rn(-q_hi, -v));
    return __fadd_rn(s, __fadd_rn(se, __fadd_rn(p_lo, fmaf(al, tt, -q_lo))));
}
__device__ __forceinline__ float2 neg2(float2 v) { return make_float2(-v.x, -v.y); }
__device__ __forceinline__ float2 step_once2(float2 ah, float2 al, float2 bh, float2 bl, float2 tt, float2 p2) {
    const float2 p_hi = __fmul2_rn(ah, tt);
    const float2 p_lo = __ffma2_rn(ah, tt, neg2(p_hi));
    const float2 q_hi = __fmul2_rn(bh, p2);
    const float2 q_lo = __ffma2_rn(bl, p2, __ffma2_rn(bh, p2, neg2(q_hi)));
    const float2 s = __fadd2_rn(p_hi, neg2(q_hi));
    const float2 v = __fadd2_rn(s, neg2(p_hi));
    const float2 se = __fadd2_rn(__fadd2_rn(p_hi, neg2(__fadd2_rn(s, neg2(v)))), __fadd2_rn(neg2(q_hi), neg2(v)));
    return __fadd2_rn(s, __fadd2_rn(se, __fadd2_rn(p_lo, __ffma2_rn(al, tt, neg2(q_lo)))));
}

// rho p + d rounded once (rho = rh + rl as float-float): TwoProduct of rh p and TwoSum with
// d, plus the remainders.  The column m = 0 of the Reinsch-modified recurrence takes it:
// the two-fma form rounds rl p + d at the magnitude of d, and near the equator that
// rounding has a mean over the sphere of ~1e-8 of P_l0 at small l, which a catalog's
// monopole (a sum growing like N) leaks through into l > 0.
__device__ __forceinline__ float sum_once(float rh, float rl, float p, float d) {
    const float ph = __fmul_rn(rh, p);
    const float pl = fmaf(rh, p, -ph);
    const float s = __fadd_rn(ph, d);
    const float v = __fadd_rn(s, -ph);
    const float se = __fadd_rn(__fadd_rn(ph, -__fadd_rn(s, -v)), __fadd_rn(d, -v));
    return __fadd_rn(s, __fadd_rn(se, fmaf(rl, p, pl)));
}
__device__ __forceinline__ float2 sum_once2(float2 rh, float2 rl, float2 p, float2 d) {
    const float2 ph = __fmul2_rn(rh, p);
    const float2 pl = __ffma2_rn(rh, p, neg2(ph));
    const float2 s = __fadd2_rn(ph, d);
    const float2 v = __fadd2_rn(s, neg2(ph));
    const float2 se = __fadd2_rn(__fadd2_rn(ph, neg2(__fadd2_rn(s, neg2(v)))), __fadd2_rn(d, neg2(v)));
    return __fadd2_rn(s, __fadd2_rn(se, __ffma2_rn(rl, p, pl)));
}

template <bool EXT, bool FULLJ, int NST, bool RS>
__global__ void __launch_bounds__(NTOT, 1) k_split_l(SplitArgs a) {
    static_assert(!EXT || RS, "the extended range takes the Reinsch-modified rows");
    constexpr uint32_t STG = sm_stage(EXT, RS);
    extern __shared__ uint8_t smem_raw[];
    uint8_t *sm = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    __shared__ uint64_t mbar[2];  // MMA completion per operand buffer
    __shared__ uint64_t sbar[NST];  // TMA completion per stage
    __shared__ uint32_t tmem_base_sh;
    __shared__ uint64_t fbar[2];   // operands of buffer b written (NTHR arrivals)
    __shared__ uint64_t gfree[NST];  // stage s read by every operand thread (NTHR arrivals)
    __shared__ int abort_sh;

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int l = a.l;
    const SplitItem item = a.items[blockIdx.x];
    const SplitCat cat = a.cats[item.cat];
    const int mb0 = item.mb0;
    const int mcount = item.mcount;
    const int nh0 = item.n0;
    const int nmax = min(NHALF, cat.nmax_l[l] - nh0);  // radial orders of this half
    const bool wrows = (nh0 == 0);                      // the first half writes the Legendre rows
    const int ncols = 2 * mcount;
    const int ncols_pad = (ncols + 15) & ~15;
    uint32_t half_cols = 32;
    while ((int)half_cols < ncols_pad) half_cols <<= 1;
    const uint32_t tcols = 2 * half_cols;  // D_tile at column 0, D_acc at column half_cols

    float4 *s_tab = reinterpret_cast<float4 *>(sm + off_tab(EXT, RS, NST));
    float4 *s_kzp = reinterpret_cast<float4 *>(sm + off_kz(EXT, RS, NST));  // n pair j: (hi n, hi n+1, lo n, lo n+1)
    float *s_js = reinterpret_cast<float *>(sm + off_js(EXT, RS, NST));
    float *s_inv = reinterpret_cast<float *>(sm + off_inv(EXT, RS, NST));
    float4 *s_coef = reinterpret_cast<float4 *>(sm + off_coef(EXT, RS, NST));  // m pair j: (A_hi x2, A_lo x2), (B_hi x2, B_lo x2)
    float4 *s_rcoef = reinterpret_cast<float4 *>(sm + off_rcoef(EXT, RS, NST));  // m pair j: (c1_hi x2, c1_lo x2), (rho_hi x2, rho_lo x2)
    const float4 *kz_row = cat.kz + (size_t)l * cat.kzw + nh0;
    const float kmax_j = nmax > 0 ? kz_row[nmax - 1].x : 0.f;  // largest k_ln / H of this half (k grows with n)
    for (int t = tid; t < 2 * a.nint; t += NTOT) s_tab[t] = a.tab[t];
    // radial orders past this half's count get k = 0 and J scale 0: their J rows are zero
    for (int t = tid; t < NHALF / 2; t += NTOT) {
        const float4 ka = 2 * t < nmax ? kz_row[2 * t] : make_float4(0.f, 0.f, 0.f, 0.f);
        const float4 kb = 2 * t + 1 < nmax ? kz_row[2 * t + 1] : make_float4(0.f, 0.f, 0.f, 0.f);
        s_kzp[t] = make_float4(ka.x, kb.x, ka.y, kb.y);
        s_js[2 * t] = ka.z;
        s_js[2 * t + 1] = kb.z;
        s_inv[2 * t] = ka.w;
        s_inv[2 * t + 1] = kb.w;
    }
    for (int t = tid; t < (mcount + 1) / 2; t += NTOT) {
        const float4 ca = a.coef[mb0 + 2 * t];
        const float4 cb = 2 * t + 1 < mcount ? a.coef[mb0 + 2 * t + 1] : make_float4(0.f, 0.f, 0.f, 0.f);
        s_coef[2 * t] = make_float4(ca.x, cb.x, ca.y, cb.y);
        s_coef[2 * t + 1] = make_float4(ca.z, cb.z, ca.w, cb.w);
        if (RS) {
            const float4 ra = a.rcoef[mb0 + 2 * t];
            const float4 rb = 2 * t + 1 < mcount ? a.rcoef[mb0 + 2 * t + 1] : make_float4(0.f, 0.f, 0.f, 0.f);
            s_rcoef[2 * t] = make_float4(ra.x, rb.x, ra.y, rb.y);
            s_rcoef[2 * t + 1] = make_float4(ra.z, rb.z, ra.w, rb.w);
        }
    }
    if (tid == 0) {
        tc05::mbar_init(&mbar[0], 1);
        tc05::mbar_init(&mbar[1], 1);
        for (int k = 0; k < NST; ++k) tc05::mbar_init(&sbar[k], 1);
        tc05::mbar_init(&fbar[0], NTHR);
        tc05::mbar_init(&fbar[1], NTHR);
        for (int k = 0; k < NST; ++k) tc05::mbar_init(&gfree[k], NTHR);
        abort_sh = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    // J rows of radial orders past this half's count (a kmax cut, or nmax < 128) are zero
    // for the whole item: zero both operand buffers' J now; warps whose 8 rows are all
    // past the count then skip J entirely
    if (!FULLJ && nmax < NHALF) {
        for (int t = tid; t < (int)(2 * SM_J / 16); t += NTOT) {
            *reinterpret_cast<uint4 *>(sm + t * 16) = make_uint4(0u, 0u, 0u, 0u);            // buffer 0
            *reinterpret_cast<uint4 *>(sm + SM_BUF + t * 16) = make_uint4(0u, 0u, 0u, 0u);  // buffer 1
        }
    }
    if (warp == 0) tc05::tmem_alloc(&tmem_base_sh, tcols);
    tc05::fence_before();
    __syncthreads();
    tc05::fence_after();
    const uint32_t tmem = tmem_base_sh;
    const uint32_t d_tile = tmem, d_acc = tmem + half_cols;

    const int64_t t0 = item.t0, t1 = item.t1;
    const int q = lane, g = warp;
    // this warp's m: quads [qb0, qb1) of the block's ceil(mcount / 4) quads of complex m, spread
    // evenly (a quad fills one 16-byte column group of each Y half: whole-chunk stores)
    const int nquads = (mcount + 3) >> 2;
    const int qb0 = (g * nquads) / NOPW, qb1 = ((g + 1) * nquads) / NOPW;
    const int mlo = 4 * qb0, mhi = min(4 * qb1, mcount);  // local m range of this warp
    const uint32_t idesc = tc05::idesc_f16_mn(128, ncols_pad);
    const int stride = cat.stride;
    const size_t set = (size_t)stride * cat.lrp;
    // the rows this level writes: P_l (and, Reinsch-modified rows, X_l)
    float *__restrict__ st0 = cat.rows + (size_t)(RS ? (l & 1) : l % 3) * set;
    float *__restrict__ xt0 = cat.rows + (size_t)(RS ? 2 + (l & 1) : 0) * set;
    // extended range: the exponent words this level writes (set by the parity of l, one word
    // for P_l and X_l)
    unsigned long long *ex0 = nullptr;
    if (EXT) ex0 = cat.rexp + (size_t)(l & 1) * cat.eset;
    float *__restrict__ partial_cta = a.partial + (size_t)blockIdx.x * 256 * 128;

    uint32_t uses0 = 0, uses1 = 0, waited0 = 0, waited1 = 0;  // commits / completed waits per buffer
    int64_t iss = 0, wtd = 0;  // stage loads issued / waited (tiles of the item, counted from t0)
    bool acc_fresh = true;   // next fold overwrites D_acc
    bool first_flush = true; // partial rows not yet written by this CTA
    int folds = 0;
    bool ok = true;

    auto wait_buf = [&](int b, uint64_t limit) -> bool {
        uint32_t &wt = b ? waited1 : waited0;
        const uint32_t us = b ? uses1 : uses0;
        while (wt < us) {
            if (!tc05::mbar_wait(&mbar[b], wt & 1, limit)) return false;
            ++wt;
        }
        return true;
    };

    // stage tile t0 + j into stage j % NST, all by one thread, completing on sbar[j % NST]: the point
    // records (one bulk copy), the rows P_{l-1}(m) and P_{l-2}(m) of this block's m in
    // 32-row TMA boxes (rows past the tensor's end arrive as zeros; slots the step does
    // not read -- the sectoral m = l of P_{l-1}, m > l-2 of P_{l-2} -- hold stale rows),
    // and (extended range) the exponent words of level l-1
    // staged rows: P_{l-1} and P_{l-2} (three-term rows) or X_{l-1} (Reinsch-modified rows);
    // descriptors 0..3 are the row sets, 4 and 5 the exponent sets
    const char *tm_r1 = cat.tmaps + 128 * (RS ? (l + 1) & 1 : (l + 2) % 3);
    const char *tm_r2 = cat.tmaps + 128 * (RS ? 2 + ((l + 1) & 1) : (l + 1) % 3);
    const char *tm_e1 = cat.tmaps + 128 * (4 + ((l + 1) & 1));
    const int nb1 = l > 0 ? (mcount + 31) >> 5 : 0;
    const int nb2 = (max(0, min(mcount, RS ? l - mb0 : l - 1 - mb0)) + 31) >> 5;
    const uint32_t stage_bytes =
        SM_STPTS + 4096u * (uint32_t)(nb1 + nb2) + ((EXT && l > 0) ? SM_STEXP : 0u);
    if (tid == 0) {  // descriptors rewritten by the host between launches: read them afresh
        tc05::tmap_acquire(tm_r1);
        tc05::tmap_acquire(tm_r2);
        if (EXT) tc05::tmap_acquire(tm_e1);
    }
    auto prefetch = [&](int64_t j) {
        const int64_t t = t0 + j;
        if (t >= t1) return;
        iss = j + 1;
        if (tid != 0) return;
        const int sidx = (int)(j % NST);
        uint8_t *stg = sm + OFF_ST + (uint32_t)sidx * STG;
        tc05::fence_proxy_async();  // earlier generic reads of this stage before the async writes
        tc05::mbar_arrive_expect_tx(&sbar[sidx], stage_bytes);
        tc05::bulk_g2s(stg + 2 * SM_STROW, cat.pts + t * KT, SM_STPTS, &sbar[sidx]);
        // 32 m (16 interleaved pairs) x 32 points per box: 16 row segments of 256 B
        for (int k = 0; k < nb1; ++k) tc05::tma_load_2d(stg + k * 4096, tm_r1, (int)(2 * KT * t), (mb0 >> 1) + 16 * k, &sbar[sidx]);
        for (int k = 0; k < nb2; ++k)
            tc05::tma_load_2d(stg + SM_STROW + k * 4096, tm_r2, (int)(2 * KT * t), (mb0 >> 1) + 16 * k, &sbar[sidx]);
        if (EXT && l > 0) tc05::tma_load_2d(stg + 2 * SM_STROW + SM_STPTS, tm_e1, mb0, (int)t, &sbar[sidx]);
    };
    // the load of tile t0 + j is the (j / NST)-th completion of its stage's barrier
    auto wait_stage = [&](int64_t j, uint64_t limit) -> bool {
        if (!tc05::mbar_wait(&sbar[j % NST], (uint32_t)((j / NST) & 1), limit)) return false;
        wtd = j + 1;
        return true;
    };

    // D_acc (+)= D_tile, by the fold warps: each its lane quadrant (warp % 4), every column group
    auto fold = [&]() {
        tc05::fence_after();
        const int qd = warp & 3;
        const uint32_t lane_off = (uint32_t)(qd * 32) << 16;
        for (int gi = 0; gi < (ncols_pad >> 4); ++gi) {
            uint32_t vt[16], va[16];
            tc05::tmem_ld16(d_tile + lane_off + gi * 16, vt);
            if (!acc_fresh) tc05::tmem_ld16(d_acc + lane_off + gi * 16, va);
            tc05::tmem_wait_ld();
            if (!acc_fresh) {
#pragma unroll
                for (int j = 0; j < 16; j += 2) {
                    const float2 sm2 = __fadd2_rn(make_float2(__uint_as_float(vt[j]), __uint_as_float(vt[j + 1])),
                                                  make_float2(__uint_as_float(va[j]), __uint_as_float(va[j + 1])));
                    vt[j] = __float_as_uint(sm2.x);
                    vt[j + 1] = __float_as_uint(sm2.y);
                }
            }
            tc05::tmem_st16(d_acc + lane_off + gi * 16, vt);
        }
        tc05::tmem_wait_st();
        acc_fresh = false;
        ++folds;
    };

    // partial[cta] (+)= D_acc / (2^s_ln 2^12) (lane n), then the next fold restarts D_acc
    auto flush = [&]() {
        tc05::fence_after();
        const int qd = warp & 3;
        const int lane_n = qd * 32 + lane;
        for (int gi = 0; gi < (ncols_pad >> 4); ++gi) {
            uint32_t v[16];
            tc05::tmem_ld16(d_acc + ((uint32_t)(qd * 32) << 16) + gi * 16, v);
            tc05::tmem_wait_ld();
            if (lane_n < nmax) {
                const float inv_scale = s_inv[lane_n];
                // all 16 reads of the running partial first (L2-resident), then the writes
                float old[16];
#pragma unroll
                for (int j = 0; j < 16; ++j) {
                    const int col = gi * 16 + j;
                    const int ml = col_m(col);
                    old[j] = (!first_flush && ml < mcount)
                                 ? __ldcg(partial_cta + (size_t)(2 * ml + col_ri(col)) * 128 + lane_n)
                                 : 0.f;
                }
#pragma unroll
                for (int j = 0; j < 16; ++j) {
                    const int col = gi * 16 + j;
                    const int ml = col_m(col);
                    if (ml < mcount)
                        __stcg(partial_cta + (size_t)(2 * ml + col_ri(col)) * 128 + lane_n,
                               __uint_as_float(v[j]) * inv_scale + old[j]);
                }
            }
        }
        first_flush = false;
        acc_fresh = true;
        folds = 0;
    };

    // roles: warps 0..15 write each tile's operands (J, Y) into the two operand buffers;
    // warps 16..19 (one per TMEM lane quadrant) fold the previous tile's tensor-core sum,
    // flush, and issue the tile's MMAs.  Hand-offs: fbar[b] operands of buffer b written,
    // mbar[b] the MMAs reading buffer b complete, gfree[s] stage s read by every operand
    // thread (it may be refilled).  Every wait is bounded; a failed one raises abort_sh.
    volatile int *abort_v = &abort_sh;
    if (warp < NTHR / 32) {
        for (int64_t jp = 0; jp + 1 < NST; ++jp) prefetch(jp);  // NST - 1 tiles ahead
        for (int64_t t = t0; t < t1; ++t) {
            const int64_t j = t - t0;
            if (*abort_v) {
                ok = false;
                break;
            }
            const int b = (int)(j & 1);
            bool okp = true;
            if (tid == 0 && j >= 1 && t + NST - 1 < t1) {  // stage (j-1) % NST last held tile j-1
                okp = tc05::mbar_wait(&gfree[(j - 1) % NST], (uint32_t)(((j - 1) / NST) & 1), a.wait_ns);
            }
            if (!okp) {
                *abort_v = 1;
                ok = false;
                break;
            }
            prefetch(j + NST - 1);
            if (!(wait_buf(b, a.wait_ns) && wait_stage(j, a.wait_ns))) {
                *abort_v = 1;
                ok = false;
                break;
            }
            const int sidx = (int)(j % NST);
            uint8_t *bufp = sm + b * SM_BUF;
            uint8_t *jhi = bufp, *jlo = bufp + SM_J, *yhi = bufp + 2 * SM_J, *ylo = bufp + 2 * SM_J + SM_Y;
            const float *stg1 = reinterpret_cast<const float *>(sm + OFF_ST + (uint32_t)sidx * STG);
            const float *stg2 = stg1 + MBLK * KT;
            const unsigned long long *stge1 = reinterpret_cast<const unsigned long long *>(
                sm + OFF_ST + (uint32_t)sidx * STG + 2 * SM_STROW + SM_STPTS);
            // this thread's point record in three 16-byte loads (at the records' 48-byte stride
            // these are free of bank conflicts, the fields one by one are not)
            const uint4 *prec = reinterpret_cast<const uint4 *>(sm + OFF_ST + (uint32_t)sidx * STG +
                                                                2 * SM_STROW + q * 48);
            const uint4 pr0 = prec[0], pr1 = prec[1], pr2 = prec[2];
            struct {
                float r_hi, r_lo, w, x_hi, x_lo, s_hi, s_lo, cphi, sphi, dr;
                unsigned long long u;
            } pt;
            pt.r_hi = __uint_as_float(pr0.x);
            pt.r_lo = __uint_as_float(pr0.y);
            pt.w = __uint_as_float(pr0.z);
            pt.x_hi = __uint_as_float(pr0.w);
            pt.x_lo = __uint_as_float(pr1.x);
            pt.s_hi = __uint_as_float(pr1.y);
            pt.s_lo = __uint_as_float(pr1.z);
            pt.cphi = __uint_as_float(pr1.w);
            pt.sphi = __uint_as_float(pr2.x);
            pt.dr = __uint_as_float(pr2.y);
            pt.u = ((unsigned long long)pr2.w << 32) | pr2.z;
            const int64_t i = t * KT + q;  // records past n are zero (w = 0, so their J is 0)
            // Reinsch-modified rows: at |cos(theta)|, the factor (-1)^l of a southern point in its weight
            const float wq = (RS && (l & 1) && (pt.u & 1ull)) ? -pt.w : pt.w;
            // ---- J tile: n = 8 g .. 8 g + 7 ----
            if constexpr (FULLJ && NOPW == 16) {
                const float2 rh2 = make_float2(pt.r_hi, pt.r_hi), rl2 = make_float2(pt.r_lo, pt.r_lo);
                const float2 w2 = make_float2(wq, wq);
                const int n0 = 8 * g;
                float2 v[4];
                const SplitPt &pc = *reinterpret_cast<const SplitPt *>(sm + OFF_ST + (uint32_t)sidx * STG +
                                                                       2 * SM_STROW + 16 * 48);
                if (kmax_j * pc.dr <= JT_TAU) {  // the same for every thread of the CTA
                    // J(n, q) = w_q sum_j c'_j dr_q^j about the tile's record-16 radius r_c:
                    // c'_j = 2^s_n k_n^j p^(j)(u0_n) / j!, p the interval polynomial, u0_n the
                    // offset of z_n = k_n r_c in its interval (float-float product)
                    float *cs = reinterpret_cast<float *>(sm + off_jt(EXT, RS, NST)) + JPW * 8 * g;
                    __syncwarp();
                    if (lane < 8) {
                        const int n = n0 + lane;
                        const float4 kk = s_kzp[n >> 1];
                        const float kx = (n & 1) ? kk.y : kk.x, ky = (n & 1) ? kk.w : kk.z;
                        const float p = __fmul_rn(pc.r_hi, kx);
                        float e = fmaf(pc.r_hi, kx, -p);
                        e = fmaf(pc.r_hi, ky, e);
                        e = fmaf(pc.r_lo, kx, e);
                        const float fl = rintf(p);
                        const float u0 = __fadd_rn(__fadd_rn(p, -fl), e);
                        const unsigned ia = min((unsigned)(int)fl, (unsigned)(a.nint - 1));
                        const float4 a0 = s_tab[2 * ia], a1 = s_tab[2 * ia + 1];
                        // Taylor shift by synthetic division: b_0..b_3 = p(u0), p'(u0), p''(u0)/2, p'''(u0)/6
                        float b0 = a0.x, b1 = a0.y, b2 = a0.z, b3 = a0.w, b4 = a1.x, b5 = a1.y;
                        const float b6 = a1.z;
                        b5 = fmaf(b6, u0, b5); b4 = fmaf(b5, u0, b4); b3 = fmaf(b4, u0, b3);
                        b2 = fmaf(b3, u0, b2); b1 = fmaf(b2, u0, b1); b0 = fmaf(b1, u0, b0);
                        b5 = fmaf(b6, u0, b5); b4 = fmaf(b5, u0, b4); b3 = fmaf(b4, u0, b3);
                        b2 = fmaf(b3, u0, b2); b1 = fmaf(b2, u0, b1);
                        b5 = fmaf(b6, u0, b5); b4 = fmaf(b5, u0, b4); b3 = fmaf(b4, u0, b3);
                        b2 = fmaf(b3, u0, b2);
                        b5 = fmaf(b6, u0, b5); b4 = fmaf(b5, u0, b4); b3 = fmaf(b4, u0, b3);
                        const float js = s_js[n];
                        const float k1 = kx * js, k2 = k1 * kx, k3 = k2 * kx;
                        // pair layout: (c0 n, c0 n+1, c1 n, c1 n+1, c2 n, c2 n+1, c3 n, c3 n+1)
                        float *o = cs + 8 * (lane >> 1) + (lane & 1);
                        o[0] = b0 * js;
                        o[2] = b1 * k1;
                        o[4] = b2 * k2;
                        o[6] = b3 * k3;
                    }
                    __syncwarp();
                    const float dq = (q == 16) ? 0.f : pt.dr;
                    const float2 d2 = make_float2(dq, dq);
    #pragma unroll
                    for (int k = 0; k < 4; ++k) {
                        const float4 ca = *reinterpret_cast<const float4 *>(cs + 8 * k);
                        const float4 cb = *reinterpret_cast<const float4 *>(cs + 8 * k + 4);
                        float2 jv = __ffma2_rn(make_float2(cb.z, cb.w), d2, make_float2(cb.x, cb.y));
                        jv = __ffma2_rn(jv, d2, make_float2(ca.z, ca.w));
                        jv = __ffma2_rn(jv, d2, make_float2(ca.x, ca.y));
                        v[k] = __fmul2_rn(jv, w2);
                    }
                } else {
    #pragma unroll
                for (int k = 0; k < 4; ++k) {
                    const int n = n0 + 2 * k;
                    const float4 kk = s_kzp[n >> 1];
                    const float2 kx = make_float2(kk.x, kk.y), ky = make_float2(kk.z, kk.w);
                    // z = r k as float-float: p + e
                    const float2 p = __fmul2_rn(rh2, kx);
                    float2 e = __ffma2_rn(rh2, kx, make_float2(-p.x, -p.y));
                    e = __ffma2_rn(rh2, ky, e);
                    e = __ffma2_rn(rl2, kx, e);
                    const float2 fl = make_float2(rintf(p.x), rintf(p.y));
                    const float2 uu = __fadd2_rn(__fadd2_rn(p, make_float2(-fl.x, -fl.y)), e);  // in [-1/2, 1/2]
                    // radii are checked on the host against the table's extent; clamp regardless
                    const unsigned ia = min((unsigned)(int)fl.x, (unsigned)(a.nint - 1));
                    const unsigned ib = min((unsigned)(int)fl.y, (unsigned)(a.nint - 1));
                    const float4 a0 = s_tab[2 * ia], a1 = s_tab[2 * ia + 1];
                    const float4 b0 = s_tab[2 * ib], b1 = s_tab[2 * ib + 1];
                    float ja = fmaf(a1.z, uu.x, a1.y), jb = fmaf(b1.z, uu.y, b1.y);
                    ja = fmaf(ja, uu.x, a1.x);
                    jb = fmaf(jb, uu.y, b1.x);
                    ja = fmaf(ja, uu.x, a0.w);
                    jb = fmaf(jb, uu.y, b0.w);
                    ja = fmaf(ja, uu.x, a0.z);
                    jb = fmaf(jb, uu.y, b0.z);
                    ja = fmaf(ja, uu.x, a0.y);
                    jb = fmaf(jb, uu.y, b0.y);
                    ja = fmaf(ja, uu.x, a0.x);
                    jb = fmaf(jb, uu.y, b0.x);
                    const float2 js = *reinterpret_cast<const float2 *>(s_js + n);
                    v[k] = __fmul2_rn(make_float2(ja, jb), __fmul2_rn(w2, js));
                }
                }
                store_split8p(jhi, jlo, tc05::mn_sw128_off(n0, q, 2), v[0], v[1], v[2], v[3]);
            }
            else {
                // fewer radial orders (a kmax cut, nmax < 128): their ceil(nmax / 2) row pairs
                // spread evenly over the operand warps (the rows past the count stay zero)
                const int npr = (nmax + 1) >> 1;
                const int jp0 = (g * npr) / NOPW, jp1 = ((g + 1) * npr) / NOPW;
                const float2 rh2 = make_float2(pt.r_hi, pt.r_hi), rl2 = make_float2(pt.r_lo, pt.r_lo);
                const float2 w2 = make_float2(wq, wq);
                const SplitPt &pc = *reinterpret_cast<const SplitPt *>(sm + OFF_ST + (uint32_t)sidx * STG +
                                                                       2 * SM_STROW + 16 * 48);
                if (kmax_j * pc.dr <= JT_TAU) {  // Taylor form about the tile's record-16 radius (as above)
                    float *cs = reinterpret_cast<float *>(sm + off_jt(EXT, RS, NST)) + JPW * 8 * g;
                    __syncwarp();
                    if (lane < 2 * (jp1 - jp0)) {  // rows past the count have k = 0, J scale 0: zero coefficients
                        const int n = 2 * jp0 + lane;
                        const float4 kk = s_kzp[n >> 1];
                        const float kx = (n & 1) ? kk.y : kk.x, ky = (n & 1) ? kk.w : kk.z;
                        const float p = __fmul_rn(pc.r_hi, kx);
                        float e = fmaf(pc.r_hi, kx, -p);
                        e = fmaf(pc.r_hi, ky, e);
                        e = fmaf(pc.r_lo, kx, e);
                        const float fl = rintf(p);
                        const float u0 = __fadd_rn(__fadd_rn(p, -fl), e);
                        const unsigned ia = min((unsigned)(int)fl, (unsigned)(a.nint - 1));
                        const float4 a0 = s_tab[2 * ia], a1 = s_tab[2 * ia + 1];
                        float b0 = a0.x, b1 = a0.y, b2 = a0.z, b3 = a0.w, b4 = a1.x, b5 = a1.y;
                        const float b6 = a1.z;
                        b5 = fmaf(b6, u0, b5); b4 = fmaf(b5, u0, b4); b3 = fmaf(b4, u0, b3);
                        b2 = fmaf(b3, u0, b2); b1 = fmaf(b2, u0, b1); b0 = fmaf(b1, u0, b0);
                        b5 = fmaf(b6, u0, b5); b4 = fmaf(b5, u0, b4); b3 = fmaf(b4, u0, b3);
                        b2 = fmaf(b3, u0, b2); b1 = fmaf(b2, u0, b1);
                        b5 = fmaf(b6, u0, b5); b4 = fmaf(b5, u0, b4); b3 = fmaf(b4, u0, b3);
                        b2 = fmaf(b3, u0, b2);
                        b5 = fmaf(b6, u0, b5); b4 = fmaf(b5, u0, b4); b3 = fmaf(b4, u0, b3);
                        const float js = s_js[n];
                        const float k1 = kx * js, k2 = k1 * kx, k3 = k2 * kx;
                        float *o = cs + 8 * (lane >> 1) + (lane & 1);
                        o[0] = b0 * js;
                        o[2] = b1 * k1;
                        o[4] = b2 * k2;
                        o[6] = b3 * k3;
                    }
                    __syncwarp();
                    const float dq = (q == 16) ? 0.f : pt.dr;
                    const float2 d2 = make_float2(dq, dq);
                    for (int jp = jp0; jp < jp1; ++jp) {
                        const float *c8 = cs + 8 * (jp - jp0);
                        const float4 ca = *reinterpret_cast<const float4 *>(c8);
                        const float4 cb = *reinterpret_cast<const float4 *>(c8 + 4);
                        float2 jv = __ffma2_rn(make_float2(cb.z, cb.w), d2, make_float2(cb.x, cb.y));
                        jv = __ffma2_rn(jv, d2, make_float2(ca.z, ca.w));
                        jv = __ffma2_rn(jv, d2, make_float2(ca.x, ca.y));
                        const float2 v = __fmul2_rn(jv, w2);
                        __half2 hh = __float22half2_rn(v);
                        const float2 hf = __half22float2(hh);
                        __half2 ll = __float22half2_rn(__fadd2_rn(v, make_float2(-hf.x, -hf.y)));
                        const uint32_t off = tc05::mn_sw128_off(2 * jp, q, 2);
                        *reinterpret_cast<__half2 *>(jhi + off) = hh;
                        *reinterpret_cast<__half2 *>(jlo + off) = ll;
                    }
                } else
                for (int jp = jp0; jp < jp1; ++jp) {
                    const int n = 2 * jp;
                    const float4 kk = s_kzp[jp];
                    const float2 kx = make_float2(kk.x, kk.y), ky = make_float2(kk.z, kk.w);
                    const float2 p = __fmul2_rn(rh2, kx);
                    float2 e = __ffma2_rn(rh2, kx, make_float2(-p.x, -p.y));
                    e = __ffma2_rn(rh2, ky, e);
                    e = __ffma2_rn(rl2, kx, e);
                    const float2 fl = make_float2(rintf(p.x), rintf(p.y));
                    const float2 uu = __fadd2_rn(__fadd2_rn(p, make_float2(-fl.x, -fl.y)), e);
                    const unsigned ia = min((unsigned)(int)fl.x, (unsigned)(a.nint - 1));
                    const unsigned ib = min((unsigned)(int)fl.y, (unsigned)(a.nint - 1));
                    const float4 a0 = s_tab[2 * ia], a1 = s_tab[2 * ia + 1];
                    const float4 b0 = s_tab[2 * ib], b1 = s_tab[2 * ib + 1];
                    float ja = fmaf(a1.z, uu.x, a1.y), jb = fmaf(b1.z, uu.y, b1.y);
                    ja = fmaf(ja, uu.x, a1.x);
                    jb = fmaf(jb, uu.y, b1.x);
                    ja = fmaf(ja, uu.x, a0.w);
                    jb = fmaf(jb, uu.y, b0.w);
                    ja = fmaf(ja, uu.x, a0.z);
                    jb = fmaf(jb, uu.y, b0.z);
                    ja = fmaf(ja, uu.x, a0.y);
                    jb = fmaf(jb, uu.y, b0.y);
                    ja = fmaf(ja, uu.x, a0.x);
                    jb = fmaf(jb, uu.y, b0.x);
                    const float2 js = *reinterpret_cast<const float2 *>(s_js + n);
                    const float2 v = __fmul2_rn(make_float2(ja, jb), __fmul2_rn(w2, js));
                    __half2 hh = __float22half2_rn(v);
                    const float2 hf = __half22float2(hh);
                    __half2 ll = __float22half2_rn(__fadd2_rn(v, make_float2(-hf.x, -hf.y)));
                    const uint32_t off = tc05::mn_sw128_off(n, q, 2);
                    *reinterpret_cast<__half2 *>(jhi + off) = hh;
                    *reinterpret_cast<__half2 *>(jlo + off) = ll;
                }
            }
            // ---- Y tile: local m = mlo .. mhi-1 of this block, in pairs (m, m+1), stored by quads ----
            if (mlo < mhi) {
                // x = cos(theta) (Reinsch-modified rows: |cos(theta)|) and eps = 1 - |cos(theta)|
                const float xh = pt.x_hi, xl = pt.x_lo, eh = pt.s_hi, el = pt.s_lo, c1 = pt.cphi, s1 = pt.sphi;
                // e^{i m phi} for the pair (m, m+1), times the readout factor 2^-88 of the scaled
                // rows (exact): seed m, one rotation by e^{i phi}; pairs then advance by
                // e^{2 i phi}.  nsm holds -sin.
                float cma, sma;
                phase_seed(pt.u, mb0 + mlo, cma, sma);
                cma *= Y_UNSCALE;
                sma *= Y_UNSCALE;
                float2 cm = make_float2(cma, fmaf(cma, c1, -sma * s1));
                float2 nsm = make_float2(-sma, -fmaf(sma, c1, cma * s1));
                // P_l of the pair (m, m + 1) at this point (m even: the pair is one float2)
                float *rowp = st0 + (size_t)((mb0 + mlo) >> 1) * 2 * stride + 2 * i;
                const float c2 = fmaf(c1, c1, -s1 * s1), s2 = 2.f * c1 * s1;
                const float2 c22 = make_float2(c2, c2), s22 = make_float2(s2, s2), ns22 = make_float2(-s2, -s2);
                const float2 xh2 = make_float2(xh, xh), xl2 = make_float2(xl, xl);
                const float2 eh2 = make_float2(eh, eh), el2 = make_float2(el, el);
                float2 yq0 = make_float2(0.f, 0.f), yq1 = yq0;  // Y (Re, Im) of the quad's first pair
    #pragma unroll
                for (int pp = 0; pp < 2 * QPW; ++pp) {
                    const int ml = mlo + 2 * pp;  // even local m
                    float2 yr = make_float2(0.f, 0.f), yi = yr;
                    if (ml < mhi) {
                        {
                            const int m = mb0 + ml;
                            float2 P;
                            if constexpr (RS) {
                                // rows P_l and X_l at |cos(theta)|.  Columns m < MR_STD
                                // take the Reinsch-modified step (X = D_l = P_l - rho_l P_{l-1}):
                                //   D_l = c1_l D_{l-1} - A_l eps P_{l-1},  P_l = rho_l P_{l-1} + D_l,
                                // in which near the poles (eps -> 0) D is small and the rounding of
                                // P_l no longer accumulates through the three-term recurrence's
                                // cancellation; columns m >= MR_STD (their points lie away from the
                                // poles) keep the three-term step, X = P_{l-1}
                                float *xrowp = rowp + (xt0 - st0);
                                if (m + 1 <= l - 1 && ml + 1 < mcount) {
                                    const float2 p1 = reinterpret_cast<const float2 *>(stg1)[(ml >> 1) * KT + q];
                                    const float2 x1 = reinterpret_cast<const float2 *>(stg2)[(ml >> 1) * KT + q];
                                    const float4 ca = s_coef[ml];
                                    // extended range: P_{l-1} and X_{l-1} share one exponent per (point, m)
                                    unsigned ea = 0, eb = 0;
                                    if (EXT) {
                                        ea = ebits(stge1[ml], q);
                                        eb = ebits(stge1[ml + 1], q);
                                    }
                                    float2 Xn;
                                    if (m >= MR_STD) {
                                        const float4 cb = s_coef[ml + 1];
                                        const float2 tt = __ffma2_rn(xh2, p1, __fmul2_rn(xl2, p1));
                                        const float2 bb = __ffma2_rn(make_float2(cb.z, cb.w), x1,
                                                                     __fmul2_rn(make_float2(cb.x, cb.y), x1));
                                        const float2 vv = __ffma2_rn(make_float2(ca.z, ca.w), tt, neg2(bb));
                                        P = __ffma2_rn(make_float2(ca.x, ca.y), tt, vv);
                                        Xn = p1;
                                    } else {
                                        const float4 ra = s_rcoef[ml], rb = s_rcoef[ml + 1];
                                        const float2 u = __ffma2_rn(eh2, p1, __fmul2_rn(el2, p1));
                                        const float2 corr = __ffma2_rn(make_float2(ra.z, ra.w), x1,
                                                                       __fmul2_rn(make_float2(-ca.z, -ca.w), u));
                                        Xn = __ffma2_rn(make_float2(ra.x, ra.y), x1,
                                                        __ffma2_rn(make_float2(-ca.x, -ca.y), u, corr));
                                        if (m == 0)
                                            P = sum_once2(make_float2(rb.x, rb.y), make_float2(rb.z, rb.w), p1, Xn);
                                        else
                                            P = __ffma2_rn(make_float2(rb.x, rb.y), p1,
                                                           __ffma2_rn(make_float2(rb.z, rb.w), p1, Xn));
                                    }
                                    if (EXT) {  // renormalise P_l and X_l together once P_l grew past 2^40 while e > 0
                                        if (ea > 0 && fabsf(P.x) > 0x1p40f) {
                                            P.x = P.x * 0x1p-64f * 0x1p-64f;
                                            Xn.x = Xn.x * 0x1p-64f * 0x1p-64f;
                                            --ea;
                                        }
                                        if (eb > 0 && fabsf(P.y) > 0x1p40f) {
                                            P.y = P.y * 0x1p-64f * 0x1p-64f;
                                            Xn.y = Xn.y * 0x1p-64f * 0x1p-64f;
                                            --eb;
                                        }
                                    }
                                    if (wrows) {
                                        *reinterpret_cast<float2 *>(rowp) = P;
                                        *reinterpret_cast<float2 *>(xrowp) = Xn;
                                    }
                                    if (EXT && wrows) {
                                        const unsigned a0 = __ballot_sync(0xffffffffu, ea & 1u);
                                        const unsigned a1 = __ballot_sync(0xffffffffu, (ea >> 1) & 1u);
                                        const unsigned b0 = __ballot_sync(0xffffffffu, eb & 1u);
                                        const unsigned b1 = __ballot_sync(0xffffffffu, (eb >> 1) & 1u);
                                        if (lane == 0) {
                                            ex0[t * cat.epitch + m] = ((unsigned long long)a1 << 32) | a0;
                                            ex0[t * cat.epitch + m + 1] = ((unsigned long long)b1 << 32) | b0;
                                        }
                                    }
                                    if (EXT) {  // values with e > 0 are below 2^-188: no contribution
                                        if (ea) P.x = 0.f;
                                        if (eb) P.y = 0.f;
                                    }
                                } else {
                                    // the sectoral m = l (the FP64 seed, X = 0), or the block's last odd m
                                    const float4 ca = s_coef[ml], cb = s_coef[ml + 1];
                                    const float4 ra = s_rcoef[ml], rb = s_rcoef[ml + 1];
                                    float pv[2];
    #pragma unroll
                                    for (int h = 0; h < 2; ++h) {
                                        const int mlh = ml + h, mh = m + h;
                                        float Pq = 0.f, Xq = 0.f;
                                        unsigned e = 0;
                                        if (mlh < mhi) {  // warp-uniform
                                            const int si = ((mlh >> 1) * KT + q) * 2 + (mlh & 1);
                                            if (l == 0) {
                                                Pq = P00_SCALED;
                                            } else if (mh == l) {
                                                Pq = stg1[si];
                                                if (EXT) e = ebits(stge1[mlh], q);
                                            } else {
                                                const float p1 = stg1[si], x1 = stg2[si];
                                                if (EXT) e = ebits(stge1[mlh], q);
                                                const float A_hi = h ? ca.y : ca.x, A_lo = h ? ca.w : ca.z;
                                                if (mh >= MR_STD) {
                                                    const float B_hi = h ? cb.y : cb.x, B_lo = h ? cb.w : cb.z;
                                                    Pq = step_once(A_hi, A_lo, B_hi, B_lo, fmaf(xh, p1, xl * p1), x1);
                                                    Xq = p1;
                                                } else {
                                                    const float c_hi = h ? ra.y : ra.x, c_lo = h ? ra.w : ra.z;
                                                    const float r_hi = h ? rb.y : rb.x, r_lo = h ? rb.w : rb.z;
                                                    const float u = fmaf(eh, p1, el * p1);
                                                    Xq = fmaf(c_hi, x1, fmaf(-A_hi, u, fmaf(c_lo, x1, -A_lo * u)));
                                                    Pq = (mh == 0) ? sum_once(r_hi, r_lo, p1, Xq)
                                                                   : fmaf(r_hi, p1, fmaf(r_lo, p1, Xq));
                                                }
                                                if (EXT && e > 0 && fabsf(Pq) > 0x1p40f) {
                                                    Pq = Pq * 0x1p-64f * 0x1p-64f;
                                                    Xq = Xq * 0x1p-64f * 0x1p-64f;
                                                    --e;
                                                }
                                            }
                                            if (wrows) {
                                                rowp[h] = Pq;
                                                xrowp[h] = Xq;
                                            }
                                            if (EXT && wrows) {
                                                const unsigned b0w = __ballot_sync(0xffffffffu, e & 1u);
                                                const unsigned b1w = __ballot_sync(0xffffffffu, (e >> 1) & 1u);
                                                if (lane == 0) ex0[t * cat.epitch + mh] = ((unsigned long long)b1w << 32) | b0w;
                                            }
                                            if (EXT && e != 0) Pq = 0.f;  // below 2^-188: no contribution
                                        }
                                        pv[h] = Pq;
                                    }
                                    P = make_float2(pv[0], pv[1]);
                                }
                            } else if (m + 1 <= l - 2 && ml + 1 < mcount) {
                                // both m take the plain three-term step: packed arithmetic
                                const float4 ca = s_coef[ml], cb = s_coef[ml + 1];
                                const float2 p1 = reinterpret_cast<const float2 *>(stg1)[(ml >> 1) * KT + q];
                                const float2 p2 = reinterpret_cast<const float2 *>(stg2)[(ml >> 1) * KT + q];
                                const float2 tt = __ffma2_rn(xh2, p1, __fmul2_rn(xl2, p1));
                                if (m == 0) {  // the m = 0 column rounded once (step_once)
                                    P = step_once2(make_float2(ca.x, ca.y), make_float2(ca.z, ca.w),
                                                   make_float2(cb.x, cb.y), make_float2(cb.z, cb.w), tt, p2);
                                } else {
                                    const float2 bb = __ffma2_rn(make_float2(cb.z, cb.w), p2,
                                                                 __fmul2_rn(make_float2(cb.x, cb.y), p2));
                                    const float2 vv =
                                        __ffma2_rn(make_float2(ca.z, ca.w), tt, make_float2(-bb.x, -bb.y));
                                    P = __ffma2_rn(make_float2(ca.x, ca.y), tt, vv);
                                }
                                if (wrows) *reinterpret_cast<float2 *>(rowp) = P;
                            } else {
                                // sectoral (m = l), m = l - 1, or the block's last odd m
                                const float4 ca = s_coef[ml], cb = s_coef[ml + 1];
                                float pv[2];
    #pragma unroll
                                for (int h = 0; h < 2; ++h) {
                                    const int mlh = ml + h, mh = m + h;
                                    float Pq = 0.f;
                                    if (mlh < mhi) {  // warp-uniform
                                        if (l == 0) {
                                            Pq = P00_SCALED;
                                        } else if (mh == l) {
                                            // the FP64 sectoral seed, rounded once by k_split_sectoral
                                            // into slot l of the P_{l-1} set
                                            Pq = stg1[((mlh >> 1) * KT + q) * 2 + (mlh & 1)];
                                        } else if (mh == l - 1) {
                                            // P_{l,l-1} = sqrt(2l+1) x P_{l-1,l-1}, rounded once
                                            const float A_hi = h ? ca.y : ca.x, A_lo = h ? ca.w : ca.z;
                                            const float p1 = stg1[((mlh >> 1) * KT + q) * 2 + (mlh & 1)];
                                            const float tt = fmaf(xh, p1, xl * p1);
                                            Pq = step_once(A_hi, A_lo, 0.f, 0.f, tt, 0.f);
                                        } else {  // m <= l - 2: one recurrence step, rounded once
                                            const float A_hi = h ? ca.y : ca.x, A_lo = h ? ca.w : ca.z;
                                            const float B_hi = h ? cb.y : cb.x, B_lo = h ? cb.w : cb.z;
                                            const float p1 = stg1[((mlh >> 1) * KT + q) * 2 + (mlh & 1)];
                                            const float p2 = stg2[((mlh >> 1) * KT + q) * 2 + (mlh & 1)];
                                            const float tt = fmaf(xh, p1, xl * p1);
                                            // rounded once (step_once); at l = 2, m = 0 P_{l-2} = P_00
                                            // is the same for every point, so the fma chain's error
                                            // would even be one constant shared by all points
                                            Pq = step_once(A_hi, A_lo, B_hi, B_lo, tt, p2);
                                        }
                                        if (wrows) rowp[h] = Pq;
                                    }
                                    pv[h] = Pq;
                                }
                                P = make_float2(pv[0], pv[1]);
                            }
                            yr = __fmul2_rn(P, cm);
                            yi = __fmul2_rn(P, nsm);
                            // e^{i (m+2) phi} = e^{i m phi} e^{2 i phi}
                            const float2 cmn = __ffma2_rn(cm, c22, __fmul2_rn(nsm, s22));
                            nsm = __ffma2_rn(nsm, c22, __fmul2_rn(cm, ns22));
                            cm = cmn;
                        }
                    }
                    if (pp & 1) {
                        // the quad of pairs pp - 1, pp: one 16-byte chunk per half (a second pair past
                        // the warp's range enters as zeros, in columns the flush never reads)
                        if (ml - 2 < mhi)
                            store_split8p(yhi, ylo, tc05::mn_sw128_off(2 * (ml - 2), q, 4), yq0, yq1, yr, yi);
                    } else {
                        yq0 = yr;
                        yq1 = yi;
                    }
                    rowp += 2 * (size_t)stride;
                }
            }
            tc05::fence_proxy_async();
            ws_arrive(&gfree[sidx]);
            if (!(a.stall && t == t0)) ws_arrive(&fbar[b]);  // the test hook withholds the first hand-off
            if (b) ++uses1; else ++uses0;
        }
        // stage loads still in flight (a loop that stopped early) land before the CTA exits
        while (wtd < iss && wait_stage(wtd, WAIT_NS)) {
        }
    } else {
        uint32_t fw0 = 0, fw1 = 0;  // fbar phases waited
        for (int64_t t = t0; t < t1; ++t) {
            const int b = (int)((t - t0) & 1);
            uint32_t &fw = b ? fw1 : fw0;
            bool okw = tc05::mbar_wait(&fbar[b], fw & 1, a.wait_ns);
            ++fw;
            if (okw && t > t0) okw = wait_buf(b ^ 1, a.wait_ns);  // the MMAs of tile t-1 (D_tile) complete
            if (!fold_vote(okw && !*abort_v)) {        // the fold warps decide together
                *abort_v = 1;
                ok = false;
                break;
            }
            if (t > t0) {
                fold();
                if (folds == FLUSH_FOLDS) flush();
            }
            tc05::fence_before();
            fold_bar();
            tc05::fence_after();
            uint8_t *bufp = sm + b * SM_BUF;
            uint8_t *jhi = bufp, *jlo = bufp + SM_J, *yhi = bufp + 2 * SM_J, *ylo = bufp + 2 * SM_J + SM_Y;
            const bool fresh_tile = ((t - t0) % FOLD_TILES == 0);  // D_tile was folded (or never used)
            if (tid == NTHR) {
                const uint32_t sj_hi = tc05::smem_u32(jhi), sj_lo = tc05::smem_u32(jlo);
                const uint32_t sy_hi = tc05::smem_u32(yhi), sy_lo = tc05::smem_u32(ylo);
                // the four small hi x lo / lo x hi products first, the two hi x hi last: the
                // tensor core rounds each MMA's sum into the FP32 accumulator, and the
                // small terms then round at their own magnitude (2^-11 of the sum), so
                // only two roundings per tile fall at the full magnitude instead of five
                uint64_t ah[2], al[2], bh[2], bl[2];
    #pragma unroll
                for (int ks = 0; ks < 2; ++ks) {
                    ah[ks] = tc05::desc_sw128(sj_hi + ks * 4096, 1024, 2048);
                    al[ks] = tc05::desc_sw128(sj_lo + ks * 4096, 1024, 2048);
                    bh[ks] = tc05::desc_sw128(sy_hi + ks * 8192, 1024, 4096);
                    bl[ks] = tc05::desc_sw128(sy_lo + ks * 8192, 1024, 4096);
                }
                tc05::mma_f16(d_tile, ah[0], bl[0], idesc, fresh_tile ? 0u : 1u);
                tc05::mma_f16(d_tile, al[0], bh[0], idesc, 1u);
                tc05::mma_f16(d_tile, ah[1], bl[1], idesc, 1u);
                tc05::mma_f16(d_tile, al[1], bh[1], idesc, 1u);
                tc05::mma_f16(d_tile, ah[0], bh[0], idesc, 1u);
                tc05::mma_f16(d_tile, ah[1], bh[1], idesc, 1u);
                tc05::commit(&mbar[b]);
            }
            if (b) ++uses1; else ++uses0;
        }
        if (ok && t1 > t0) {
            const int lb = (int)((t1 - 1 - t0) & 1);
            ok = fold_vote(wait_buf(lb, a.wait_ns));
            if (ok) {
                fold();
                flush();
            }
        }
        if (ok) ok = fold_vote(wait_buf(0, a.wait_ns) && wait_buf(1, a.wait_ns));
        if (!ok) {
            // MMAs already issued land before TMEM is released (bounded by the 1 s
            // drain limit, not by the possibly shortened pipeline limit)
            wait_buf(0, WAIT_NS);
            wait_buf(1, WAIT_NS);
            *abort_v = 1;
        }
    }
    if (!ok && (tid == 0 || tid == NTHR)) *a.err = CATANA_ERR_CUDA;
    // an empty slab still owns partial rows: write zeros so the reduction sees them
    if (t0 >= t1) {
        for (int t = tid; t < ncols * 128; t += NTOT) partial_cta[t] = 0.f;
    }
    tc05::fence_before();
    __syncthreads();
    tc05::fence_after();
    if (warp == 0) tc05::tmem_dealloc(tmem, tcols);
}

// Sectoral seeds (one warp per tile, lane = point): P_ll 2^100 advanced in FP64,
// P_ll = a_l s P_{l-1,l-1} from the FP32 value of P_00 (the row every m = 0 step
// uses, so the m = 0 recurrence sees one consistent P_00), rounded once and stored in
// slot m = l of the P_{l-1} row set for l = 1 .. lmax-1.  Extended range: in the
// frame of the running 2-bit exponent (stored value P 2^100 2^(128 e), e raised when
// the value drops below 2^-40, 0 below 2^-520), with the exponent word written too.
// mode bit 0: Reinsch-modified rows (sets by the parity of l, records carrying 1 - |cos(theta)|);
// bit 1: extended range (exponent words; always with bit 0)
__global__ void k_split_sectoral(const SplitCat *cats, int cat, int lmax, const double *__restrict__ asect,
                                 int64_t ntiles, int mode) {
    const bool rs = (mode & 1) != 0, ext = (mode & 2) != 0;
    const SplitCat c = cats[cat];
    const int64_t t = blockIdx.x * (int64_t)(blockDim.x >> 5) + (threadIdx.x >> 5);
    if (t >= ntiles) return;  // warp-uniform
    const int q = threadIdx.x & 31;
    const int64_t i = t * KT + q;
    const SplitPt &pt = c.pts[i];
    // sin(theta): stored (extended range), or from eps = 1 - |cos(theta)| as sqrt(eps (2 - eps))
    const double sv = (double)pt.s_hi + (double)pt.s_lo;
    const double s = rs ? sqrt(sv * (2.0 - sv)) : sv;
    const size_t set = (size_t)c.stride * c.lrp;
    float *rt = c.rows + 2 * i;  // this point in the pair-interleaved rows
    double P = (double)P00_SCALED;
    unsigned e = 0;
    for (int l = 1; l < lmax; ++l) {
        P = asect[l] * s * P;
        const int k = rs ? (l + 1) & 1 : (l + 2) % 3;  // the set of P_{l-1} (and of its exponent words)
        float v;
        if (ext) {
            double f = P;
            for (unsigned j = 0; j < e; ++j) f *= 0x1p128;
            v = (float)f;
            if (fabsf(v) < 0x1p-40f) {
                if (e < 3) {
                    ++e;
                    v = (float)(f * 0x1p128);
                } else {
                    v = 0.f;  // below 2^-520: no contribution within lmax
                }
            }
            const unsigned b0 = __ballot_sync(0xffffffffu, e & 1u), b1 = __ballot_sync(0xffffffffu, (e >> 1) & 1u);
            if (q == 0) c.rexp[(size_t)k * c.eset + t * c.epitch + l] = ((unsigned long long)b1 << 32) | b0;
        } else {
            v = (float)P;
        }
        rt[(size_t)k * set + (size_t)(l >> 1) * 2 * c.stride + (l & 1)] = v;
    }
}

// One catalog's reduction at one level: its items are ordered block-major, then slab.
struct SplitRed {
    int item0, nslabs, mblk, nmax_l, kzw, nhalves;  // items: block-major, then half, then slab
    double2 *fl;            // f accumulator block of l: [m][kzw]
    const double *kln_row;  // k_ln row l (kzw entries)
};

// f[l][m][n] += k_ln[n] * sum_slab partial[item(m / mblk, slab)][2 (m % mblk) + ri][n]
// (FP64, slab order); blockIdx.y selects the catalog.
__global__ void k_split_reduce(const float *__restrict__ partial, int lp1, const SplitRed *__restrict__ reds) {
    const SplitRed r = reds[blockIdx.y];
    const int t = blockIdx.x * blockDim.x + threadIdx.x;  // (m, n)
    if (t >= lp1 * r.nmax_l) return;
    const int m = t / r.nmax_l, n = t - m * r.nmax_l;
    const int blk = m / r.mblk, ml = m - blk * r.mblk;
    const int hf = n / NHALF, nl = n - hf * NHALF;
    double sr = 0.0, si = 0.0;
    for (int sl = 0; sl < r.nslabs; ++sl) {
        const float *p = partial + (size_t)(r.item0 + (blk * r.nhalves + hf) * r.nslabs + sl) * 256 * 128;
        sr += (double)p[(size_t)(2 * ml) * 128 + nl];
        si += (double)p[(size_t)(2 * ml + 1) * 128 + nl];
    }
    const double k = r.kln_row[n];
    double2 *o = r.fl + (size_t)m * r.kzw + n;
    double2 v = *o;
    v.x += k * sr;
    v.y += k * si;
    *o = v;
}

// Point preparation, in radius-sorted order: float-float r, cos(theta), sin(theta);
// e^{i phi} in FP32; the 64-bit phase fraction; FP32 weights.  Flags radii that are
// negative or not finite.  Records past n (padding to whole tiles) are zeroed.
// Each record also carries dr = r - r_c, r_c the radius of its tile's record 16 (0 if
// that record is padding), and record 16 carries the tile's max |dr| instead: the J
// operand of a tile whose radii lie close together comes from a Taylor expansion
// about r_c (k_split_l).  One warp per tile (blockDim a multiple of 32).
// Reinsch-modified rows (`plain` set): the rows are evaluated at
// |cos(theta)|, since P_lm(-x) = (-1)^(l+m) P_lm(x): a point of the southern hemisphere
// takes phi + pi (the factor (-1)^m of the phase), bit 0 of its phase fraction records
// the hemisphere and k_split_l applies (-1)^l through its J weight.  The record then
// carries 1 - |cos(theta)| = 2 sin^2(theta / 2) (north) or 2 cos^2(theta / 2) (south),
// exact to a relative 1e-16 right up to the poles, in place of sin(theta).
template <typename T>
__global__ void k_split_prep(const T *__restrict__ pts, const T *__restrict__ w,
                             const uint32_t *__restrict__ perm, int64_t n, int64_t npad, SplitPt *out, int *err,
                             int plain) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i - (threadIdx.x & 31) >= npad) return;  // whole warps (npad is a multiple of 32)
    const int64_t ic = (i & ~(int64_t)31) + 16;
    const double rc = ic < n ? (double)pts[3 * (int64_t)perm[ic]] : 0.0;
    const double dr = i < n ? (double)pts[3 * (int64_t)perm[i]] - rc : 0.0;
    float dmax = (float)fabs(dr);
    for (int o = 16; o > 0; o >>= 1) dmax = fmaxf(dmax, __shfl_xor_sync(0xffffffffu, dmax, o));
    SplitPt o;
    if (i >= n) {
        o.r_hi = o.r_lo = o.w = o.x_hi = o.x_lo = o.s_hi = o.s_lo = o.cphi = o.sphi = 0.f;
        o.dr = (threadIdx.x & 31) == 16 ? dmax : 0.f;
        o.u = 0ull;
        out[i] = o;
        return;
    }
    const int64_t j = perm[i];
    const double r = (double)pts[3 * j], th = (double)pts[3 * j + 1], ph = (double)pts[3 * j + 2];
    if (!(r >= 0.0) || !isfinite(r)) *err = CATANA_ERR_DOMAIN;
    double st, ct, sp, cp;
    sincos(th, &st, &ct);
    sincos(ph, &sp, &cp);
    o.r_hi = (float)r;
    o.r_lo = (float)(r - (double)o.r_hi);
    const bool south = plain && ct < 0.0;
    double xv = ct, sv = st;
    if (plain) {
        double sh, ch;
        sincos(0.5 * th, &sh, &ch);
        xv = fabs(ct);
        sv = south ? 2.0 * ch * ch : 2.0 * sh * sh;  // 1 - |cos(theta)|
    }
    o.x_hi = (float)xv;
    o.x_lo = (float)(xv - (double)o.x_hi);
    o.s_hi = (float)sv;
    o.s_lo = (float)(sv - (double)o.s_hi);
    o.cphi = (float)(south ? -cp : cp);
    o.sphi = (float)(south ? -sp : sp);
    o.dr = (threadIdx.x & 31) == 16 ? dmax : (float)dr;
    double f = ph * 0.15915494309189533577;  // phi / 2pi
    f -= floor(f);
    const double scaled = ldexp(f, 64);
    unsigned long long u = scaled >= 18446744073709551615.0 ? 0ull : (unsigned long long)scaled;
    if (south) u += 0x8000000000000000ull;  // + half a turn
    o.u = (u & ~1ull) | (south ? 1ull : 0ull);  // bit 0 (2^-64 of a turn): the hemisphere
    o.w = w ? (float)w[j] : 1.0f;
    out[i] = o;
}

// radius keys for the sort: 16-bit quantisation of r / max_r, and the identity payload
template <typename T>
__global__ void k_split_keys(const T *__restrict__ pts, int64_t n, double inv_rmax, uint32_t *keys,
                             uint32_t *vals) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double q = (double)pts[3 * i] * inv_rmax * 65536.0;
    keys[i] = q >= 65535.0 ? 65535u : (q > 0.0 ? (uint32_t)q : 0u);
    vals[i] = (uint32_t)i;
}

// max(r) and max(|w|) as IEEE bit patterns of non-negative doubles
template <typename T>
__global__ void k_split_maxes(const T *__restrict__ pts, const T *__restrict__ w, int64_t n,
                              unsigned long long *out) {
    double mr = 0.0, mw = w ? 0.0 : 1.0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double r = (double)pts[3 * i];
        if (r > mr) mr = r;
        if (w) {
            const double a = fabs((double)w[i]);
            if (a > mw) mw = a;
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        mr = fmax(mr, __shfl_xor_sync(0xffffffffu, mr, o));
        mw = fmax(mw, __shfl_xor_sync(0xffffffffu, mw, o));
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMax(&out[0], (unsigned long long)__double_as_longlong(mr));
        atomicMax(&out[1], (unsigned long long)__double_as_longlong(mw));
    }
}

// j_l at the 6 Chebyshev nodes of every interval, all l at once per node (FP64).
// Chebyshev node k of the degree-TDEG interpolant on an interval, as an offset in [-1/2, 1/2]
__host__ __device__ inline double cheb_node(int k) { return 0.5 * cos((2.0 * k + 1.0) * kPi / (2.0 * (TDEG + 1))); }

__global__ void k_split_nodes(int lmax, int nint, double *vals /* [node][lmax] */) {
    const int node = blockIdx.x * blockDim.x + threadIdx.x;
    if (node >= nint * (TDEG + 1)) return;
    const int j = node / (TDEG + 1), k = node - (TDEG + 1) * j;
    const double z = H * (j + cheb_node(k));  // interval j is centred on z = j H
    double buf[SPLIT_LMAX_EXT + 1];
    sbessel_jl_all(lmax, fabs(z), buf);
    for (int l = 0; l < lmax; ++l)  // j_l(-z) = (-1)^l j_l(z): the first interval straddles 0
        vals[(size_t)node * lmax + l] = (z < 0.0 && (l & 1)) ? -buf[l] : buf[l];
}

// monomial coefficients in u in [-1/2, 1/2] of the interpolant through the nodes
__global__ void k_split_coefs(int lmax, int nint, const double *vals, const double *vinv,
                              float4 *tab /* [l][nint][2] */) {
    constexpr int NC = TDEG + 1;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= lmax * nint) return;
    const int l = t / nint, j = t - l * nint;
    double y[NC], c[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int k = 0; k < NC; ++k) y[k] = vals[(size_t)(NC * j + k) * lmax + l];
    for (int r = 0; r < NC; ++r) {
        double s = 0.0;
        for (int k = 0; k < NC; ++k) s += vinv[NC * r + k] * y[k];
        c[r] = s;
    }
    float4 *o = tab + ((size_t)l * nint + j) * 2;
    o[0] = make_float4((float)c[0], (float)c[1], (float)c[2], (float)c[3]);
    o[1] = make_float4((float)c[4], (float)c[5], (float)c[6], (float)c[7]);
}

void split_ff(double v, float &hi, float &lo) {
    hi = (float)v;
    lo = (float)(v - (double)hi);
}

// inverse of the Vandermonde matrix V[k][r] = u_k^r at the Chebyshev nodes (FP64,
// Gauss-Jordan with partial pivoting), row-major NC x NC
std::vector<double> cheb_vandermonde_inverse() {
    constexpr int NC = TDEG + 1;
    double A[NC][2 * NC];
    for (int k = 0; k < NC; ++k) {
        const double tk = cheb_node(k);
        double p = 1.0;
        for (int r = 0; r < NC; ++r) {
            A[k][r] = p;
            p *= tk;
        }
        for (int r = 0; r < NC; ++r) A[k][NC + r] = (r == k) ? 1.0 : 0.0;
    }
    for (int col = 0; col < NC; ++col) {
        int piv = col;
        for (int r = col + 1; r < NC; ++r)
            if (std::fabs(A[r][col]) > std::fabs(A[piv][col])) piv = r;
        for (int c = 0; c < 2 * NC; ++c) std::swap(A[col][c], A[piv][c]);
        const double d = A[col][col];
        for (int c = 0; c < 2 * NC; ++c) A[col][c] /= d;
        for (int r = 0; r < NC; ++r)
            if (r != col) {
                const double f = A[r][col];
                for (int c = 0; c < 2 * NC; ++c) A[r][c] -= f * A[col][c];
            }
    }
    std::vector<double> inv(NC * NC);
    for (int r = 0; r < NC; ++r)
        for (int k = 0; k < NC; ++k) inv[NC * r + k] = A[r][NC + k];
    return inv;
}

}  // namespace

// ---------------------------------------------------------------------------
// Host side: a plan of (catalog, level) work items.
// ---------------------------------------------------------------------------
namespace {

struct CatPlan {
    SplitCatInput in;
    double max_r = 0.0, max_w = 1.0;
    std::vector<double> kh;     // k_ln row-major [l][nmax]
    std::vector<int> nmax_l;    // radial orders kept at each l (kmax cut)
    int64_t stride = 0, ntiles = 0;
};

size_t al256(size_t b) { return (b + 255) & ~size_t(255); }

// j_l tables for l < lmax over nint intervals (cached; a larger cached table serves)
catana_status_t ensure_split_tables(DeviceContext *ctx, int lmax, int nint, cudaStream_t st) {
    SplitCache &C = ctx->split_cache;
    if (C.lmax >= lmax && C.nint >= nint && C.lmax == (int)C.maxj.size()) return CATANA_OK;
    lmax = std::max(lmax, C.lmax);
    nint = std::max(nint, C.nint);
    const size_t tab_bytes = (size_t)lmax * nint * 2 * sizeof(float4);
    const size_t coef_bytes = (size_t)lmax * (lmax + 1) / 2 * sizeof(float4);
    // [j_l tables][(A, B) per (l, m)][(c1, rho) per (l, m): the Reinsch-modified step]
    CG_CUDA_TRY(ctx->split_tab.ensure(tab_bytes + 2 * coef_bytes + 1024));
    constexpr int NC = TDEG + 1;
    const size_t vbytes = (size_t)nint * NC * lmax * sizeof(double);
    DevBuf tmp;
    CG_CUDA_TRY(tmp.ensure(vbytes + NC * NC * sizeof(double)));
    double *vals = tmp.as<double>();
    double *vinv = vals + (size_t)nint * NC * lmax;
    std::vector<double> vi = cheb_vandermonde_inverse();
    CG_CUDA_TRY(cudaMemcpyAsync(vinv, vi.data(), NC * NC * sizeof(double), cudaMemcpyHostToDevice, st));
    k_split_nodes<<<ceil_div(nint * NC, 64), 64, 0, st>>>(lmax, nint, vals);
    count_launch();
    CG_CUDA_TRY(cudaGetLastError());
    float4 *tab = ctx->split_tab.as<float4>();
    k_split_coefs<<<ceil_div((int64_t)lmax * nint, 128), 128, 0, st>>>(lmax, nint, vals, vinv, tab);
    count_launch();
    CG_CUDA_TRY(cudaGetLastError());
    std::vector<float4> co((size_t)lmax * (lmax + 1) / 2), ro(co.size(), make_float4(0.f, 0.f, 0.f, 0.f));
    // Reinsch-modified step of column m: rho_l = Pt_lm(1) / Pt_{l-1,m}(1) (Pt = P / sin^m),
    // rho_{m+1} = A_{m+1,m}, rho_l = A_l - B_l / rho_{l-1}; c1_l = A_l - rho_l = B_l / rho_{l-1}
    for (int m = 0; m + 1 < lmax; ++m) {
        long double rho = 0.0L;
        for (int l = m + 1; l < lmax; ++l) {
            const long double dl = l, dl1 = l - 1, mm = (long double)m * m;
            long double A, B;
            if (l == m + 1) {
                A = sqrtl(2.0L * l + 1.0L);
                B = 0.0L;
            } else {
                A = sqrtl((4.0L * dl * dl - 1.0L) / (dl * dl - mm));
                B = A * sqrtl((dl1 * dl1 - mm) / (4.0L * dl1 * dl1 - 1.0L));
            }
            const long double rn = (l == m + 1) ? A : A - B / rho;
            const long double c1 = (l == m + 1) ? 0.0L : B / rho;
            float ch, cl, rh, rl;
            split_ff((double)c1, ch, cl);
            split_ff((double)rn, rh, rl);
            ro[(size_t)l * (l + 1) / 2 + m] = make_float4(ch, cl, rh, rl);
            rho = rn;
        }
    }
    for (int l = 0; l < lmax; ++l)
        for (int m = 0; m <= l; ++m) {
            double A = 0.0, B = 0.0;
            if (l >= 1 && m == l) {
                A = -std::sqrt((2.0 * l + 1.0) / (2.0 * l));
            } else if (l >= 1 && m == l - 1) {
                A = std::sqrt(2.0 * l + 1.0);
            } else if (l >= 2) {
                const double dl = l, dl1 = l - 1, mm = (double)m * m;
                const double aa = std::sqrt((4.0 * dl * dl - 1.0) / (dl * dl - mm));
                const double bb = std::sqrt((dl1 * dl1 - mm) / (4.0 * dl1 * dl1 - 1.0));
                A = aa;
                B = aa * bb;
            }
            float ah, al, bh, bl;
            split_ff(A, ah, al);
            split_ff(B, bh, bl);
            co[(size_t)l * (l + 1) / 2 + m] = make_float4(ah, al, bh, bl);
        }
    CG_CUDA_TRY(cudaMemcpyAsync(reinterpret_cast<char *>(tab) + tab_bytes, co.data(), coef_bytes,
                                cudaMemcpyHostToDevice, st));
    CG_CUDA_TRY(cudaMemcpyAsync(reinterpret_cast<char *>(tab) + tab_bytes + coef_bytes, ro.data(), coef_bytes,
                                cudaMemcpyHostToDevice, st));
    C.maxj.assign(lmax, 1.0);
    C.zpeak.assign(lmax, 0.0);
    for (int l = 1; l < lmax; ++l) {  // largest |j_l|: its first maximum, z ~ l + 0.8 l^(1/3)
        double mj = 0.0, zp = 0.0;
        const double zc = l + 0.8 * std::cbrt((double)l);
        for (int q = -200; q <= 400; ++q) {
            const double z = zc + 0.02 * q;
            if (z <= 0) continue;
            const double v = std::fabs(sbessel_jl(l, z));
            if (v > mj) {
                mj = v;
                zp = z;
            }
        }
        C.maxj[l] = 1.05 * mj;
        C.zpeak[l] = zp - 0.05;  // j_l increases monotonically below this
    }
    CG_CUDA_TRY(cudaStreamSynchronize(st));
    tmp.release();
    C.lmax = lmax;
    C.nint = nint;
    return CATANA_OK;
}

// words of one exponent set: [tile][lmax rounded up to even] plus a pad word pair
// (16-byte copies of an odd m count read one word past the block)
int64_t exp_set_words(const CatPlan &P) { return P.ntiles * ((P.in.lmax + 1) & ~1) + 2; }

// cuTensorMapEncodeTiled through the runtime's driver entry point (no libcuda link)
PFN_cuTensorMapEncodeTiled_v12000 tmap_encoder() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    if (!fn) {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    }
    return fn;
}

// 2-D row-major tensor [d1][d0] at `base` (row pitch `pitch` bytes), box b0 x b1
bool tmap_2d(CUtensorMap *m, CUtensorMapDataType dt, void *base, uint64_t d0, uint64_t d1, uint64_t pitch, uint32_t b0,
             uint32_t b1) {
    PFN_cuTensorMapEncodeTiled_v12000 enc = tmap_encoder();
    if (!enc) return false;
    const cuuint64_t dims[2] = {d0, d1};
    const cuuint64_t strides[1] = {pitch};
    const cuuint32_t box[2] = {b0, b1};
    const cuuint32_t es[2] = {1, 1};
    return enc(m, dt, 2, base, dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
               CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// autotune cache key: catalog count, sizes and multipoles of a group
std::string tune_key(const std::vector<CatPlan> &cats, int c0, int c1) {
    std::string k = std::to_string(c1 - c0);
    for (int c = c0; c < c1; ++c) {
        k += ':';
        k += std::to_string((cats[c].in.n + 4095) / 4096);
        k += '/';
        k += std::to_string(cats[c].in.lmax);
    }
    return k;
}

}  // namespace

std::atomic<uint64_t> g_split_stall_ns{0};

catana_status_t split_run(DeviceContext *ctx, std::vector<SplitCatInput> &cats_in, bool use_graph,
                          double waves, int mblk_cap, int *err_dev, cudaStream_t st) {
    if (mblk_cap != 64) mblk_cap = MBLK;
    // every catalog of a call carries the same flags
    const bool accurate = !cats_in.empty() && cats_in.front().accurate;
    std::vector<CatPlan> cats;
    for (auto &c : cats_in) {
        if (c.lmax > SPLIT_LMAX_EXT || c.nmax > SPLIT_NMAX) {
            set_error("the split form supports lmax <= 512 and nmax <= 256");
            return CATANA_ERR_ARG;
        }
        if (c.n <= 0 || c.lmax == 0 || c.nmax == 0) continue;
        if (c.n > (int64_t)0xFFFFFFF0ll) {
            set_error("the split form takes at most 2^32 - 16 points per catalog");
            return CATANA_ERR_ARG;
        }
        CatPlan p;
        p.in = c;
        cats.push_back(p);
    }
    if (cats.empty()) return CATANA_OK;
    // the test hook (catana_gpu_test_split_stall) arms one run
    const uint64_t stall_ns = g_split_stall_ns.exchange(0);
    if (!ctx->attr_split) {
        void (*const kerns[])(SplitArgs) = {
            k_split_l<false, true, 2, false>, k_split_l<false, false, 2, false>, k_split_l<false, true, 3, false>,
            k_split_l<false, false, 3, false>, k_split_l<false, true, 2, true>,  k_split_l<false, false, 2, true>,
            k_split_l<false, true, 3, true>,  k_split_l<false, false, 3, true>,  k_split_l<true, true, 2, true>,
            k_split_l<true, false, 2, true>};
        for (auto kf : kerns)
            CG_CUDA_TRY(cudaFuncSetAttribute(kf, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM_LIMIT));
        ctx->attr_split = true;
    }
    // ---- extents: max r and max |w| per catalog (one synchronisation) ----
    const int nc = (int)cats.size();
    CG_CUDA_TRY(ctx->cat_scratch.ensure((size_t)16 * nc));
    unsigned long long *mx = ctx->cat_scratch.as<unsigned long long>();
    // the workspace is shared by every stream that runs the split form on this device
    if (!ctx->split_ws_event) CG_CUDA_TRY(cudaEventCreateWithFlags(&ctx->split_ws_event, cudaEventDisableTiming));
    else CG_CUDA_TRY(cudaStreamWaitEvent(st, ctx->split_ws_event, 0));
    bool need = false;
    for (auto &P : cats) need |= (P.in.max_r < 0.0 || P.in.max_w < 0.0);
    std::vector<unsigned long long> mxh(2 * nc, 0ull);
    if (need) {
        CG_CUDA_TRY(cudaMemsetAsync(mx, 0, (size_t)16 * nc, st));
        for (int c = 0; c < nc; ++c) {
            const int64_t n = cats[c].in.n;
            const int g = (int)std::min<int64_t>(4 * ctx->sm_count, ceil_div(n, 256));
            if (cats[c].in.pts32)
                k_split_maxes<float><<<g, 256, 0, st>>>(cats[c].in.pts32, cats[c].in.w32, n, mx + 2 * c);
            else
                k_split_maxes<double><<<g, 256, 0, st>>>(cats[c].in.pts, cats[c].in.w, n, mx + 2 * c);
            count_launch();
        }
        CG_CUDA_TRY(cudaGetLastError());
        CG_CUDA_TRY(cudaMemcpyAsync(mxh.data(), mx, (size_t)16 * nc, cudaMemcpyDeviceToHost, st));
        CG_CUDA_TRY(cudaStreamSynchronize(st));
    }
    int lmax_all = 0;
    double zmax = 0.0;
    for (int c = 0; c < nc; ++c) {
        CatPlan &P = cats[c];
        memcpy(&P.max_r, &mxh[2 * c], 8);
        memcpy(&P.max_w, &mxh[2 * c + 1], 8);
        if (P.in.max_r >= 0.0) P.max_r = P.in.max_r;  // extents given by the caller
        if (P.in.max_w >= 0.0) P.max_w = P.in.max_w;
        if (!(P.max_w > 0.0)) P.max_w = 1.0;
        const int L = P.in.lmax, M = P.in.nmax;
        P.kh.resize((size_t)L * M);
        kln_table(L, M, P.in.rmax, P.kh.data());
        P.nmax_l.assign(L, M);
        for (int l = 0; l < L; ++l) {
            int k = M;
            if (P.in.kmax > 0.0) {
                k = 0;
                while (k < M && P.kh[(size_t)l * M + k] <= P.in.kmax) ++k;
            }
            P.nmax_l[l] = k;
            if (k > 0) zmax = std::max(zmax, P.kh[(size_t)l * M + k - 1] * P.max_r);
        }
        lmax_all = std::max(lmax_all, L);
        P.stride = (P.in.n + 31) / 32 * 32;
        P.ntiles = (P.in.n + KT - 1) / KT;
    }
    const int nint = (int)std::ceil(zmax / H) + 1;
    if (nint > NINT_MAX) {
        set_error("split form: k_ln * max(r) exceeds the resident j_l table (max r beyond rmax?)");
        return CATANA_ERR_DOMAIN;
    }
    catana_status_t s = ensure_split_tables(ctx, lmax_all, nint, st);
    if (s != CATANA_OK) return s;
    const int nint_tab = ctx->split_cache.nint, lmax_tab = ctx->split_cache.lmax;
    float4 *tab = ctx->split_tab.as<float4>();
    const float4 *coef_d =
        reinterpret_cast<const float4 *>(reinterpret_cast<char *>(tab) + (size_t)lmax_tab * nint_tab * 2 * sizeof(float4));

    // ---- groups of catalogs whose Legendre rows fit the budget ----
    const double row_budget = 48e9;
    std::vector<std::pair<int, int>> groups;  // [begin, end)
    {
        int b = 0;
        double acc = 0.0;
        for (int c = 0; c < nc; ++c) {
            const double need = 4.0 * cats[c].stride * ((cats[c].in.lmax + 1) & ~1) * 4.0;
            bool shared = false;  // pieces of one catalog share f: never in one level launch
            for (int q = b; q < c; ++q) shared |= (cats[q].in.f_acc == cats[c].in.f_acc);
            if (c > b && (acc + need > row_budget || shared)) {
                groups.push_back({b, c});
                b = c;
                acc = 0.0;
            }
            acc += need;
        }
        groups.push_back({b, nc});
    }
    for (auto &gr : groups) {
        const int c0 = gr.first, c1 = gr.second, gn = c1 - c0;
        int lmax_g = 0;
        for (int c = c0; c < c1; ++c) lmax_g = std::max(lmax_g, cats[c].in.lmax);
        const bool ext = lmax_g > SPLIT_LMAX;  // extended-range rows (2-bit exponents)
        // row sets: Reinsch-modified rows P_l, X_l by the parity of l (X = D or P_{l-1});
        // three-term rows P_l, P_{l-1}, P_{l-2} rotating
        // Reinsch-modified rows: with CATANA_SPLIT_ACCURATE, and always in the extended range
        // (there the three-term rows lose a few 1e-6 for points near a pole)
        const bool rs = accurate || ext;
        const int nsets = rs ? 4 : 3;
        // three stages (tiles staged two ahead) where shared memory allows: plain rows and a
        // table of at most ~750 intervals; otherwise two
        const int nst = (!ext && smem_bytes(false, rs, 3, nint) <= SMEM_LIMIT) ? 3 : 2;
        const uint32_t smem = smem_bytes(ext, rs, nst, nint);
        // kernel per level: extended-range rows above lmax 256; the full-J layout when every
        // item of the level has 128 radial orders in its half
        auto kern_for = [&](bool full) {
            if (ext) return full ? k_split_l<true, true, 2, true> : k_split_l<true, false, 2, true>;
            if (rs) {
                if (nst == 3) return full ? k_split_l<false, true, 3, true> : k_split_l<false, false, 3, true>;
                return full ? k_split_l<false, true, 2, true> : k_split_l<false, false, 2, true>;
            }
            if (nst == 3) return full ? k_split_l<false, true, 3, false> : k_split_l<false, false, 3, false>;
            return full ? k_split_l<false, true, 2, false> : k_split_l<false, false, 2, false>;
        };
        // workspace: per catalog records + rows (+ exponents); sort scratch sized for the largest
        int64_t smax = 0;
        size_t ws_bytes = 0;
        std::vector<size_t> off_pts(gn), off_rows(gn), off_exp(gn);
        for (int c = c0; c < c1; ++c) smax = std::max(smax, cats[c].stride);
        const size_t keyb = al256((size_t)smax * 4), histb = al256((size_t)256 * ((smax + 4095) / 4096 + 1) * 4);
        ws_bytes = 4 * keyb + histb;
        for (int c = c0; c < c1; ++c) {
            off_pts[c - c0] = ws_bytes;
            ws_bytes += al256((size_t)cats[c].stride * sizeof(SplitPt));
            off_rows[c - c0] = ws_bytes;
            ws_bytes += al256((size_t)nsets * cats[c].stride * ((cats[c].in.lmax + 1) & ~1) * sizeof(float));
            off_exp[c - c0] = ws_bytes;
            if (ext) ws_bytes += al256((size_t)2 * exp_set_words(cats[c]) * sizeof(unsigned long long));
        }
        CG_CUDA_TRY(ctx->split_ws.ensure(ws_bytes));
        char *ws = ctx->split_ws.as<char>();
        uint32_t *keys = reinterpret_cast<uint32_t *>(ws), *perm = reinterpret_cast<uint32_t *>(ws + keyb);
        uint32_t *tk = reinterpret_cast<uint32_t *>(ws + 2 * keyb), *tv = reinterpret_cast<uint32_t *>(ws + 3 * keyb);
        uint32_t *hist = reinterpret_cast<uint32_t *>(ws + 4 * keyb);
        // ---- per catalog: radius sort and point records ----
        for (int c = c0; c < c1; ++c) {
            CatPlan &P = cats[c];
            const int64_t n = P.in.n;
            SplitPt *spts = reinterpret_cast<SplitPt *>(ws + off_pts[c - c0]);
            const double inv_r = P.max_r > 0.0 ? 1.0 / P.max_r : 0.0;
            if (P.in.pts32)
                k_split_keys<float><<<ceil_div(n, 256), 256, 0, st>>>(P.in.pts32, n, inv_r, keys, perm);
            else
                k_split_keys<double><<<ceil_div(n, 256), 256, 0, st>>>(P.in.pts, n, inv_r, keys, perm);
            count_launch();
            CG_CUDA_TRY(cudaGetLastError());
            s = radix_sort_pairs(keys, perm, tk, tv, n, 16, hist, st);
            if (s != CATANA_OK) return s;
            const int64_t npad = P.ntiles * KT;
            if (P.in.pts32)
                k_split_prep<float><<<ceil_div(npad, 256), 256, 0, st>>>(P.in.pts32, P.in.w32, perm, n, npad, spts,
                                                                         err_dev, rs ? 1 : 0);
            else
                k_split_prep<double><<<ceil_div(npad, 256), 256, 0, st>>>(P.in.pts, P.in.w, perm, n, npad, spts,
                                                                          err_dev, rs ? 1 : 0);
            count_launch();
            CG_CUDA_TRY(cudaGetLastError());
        }
        // ---- plan tables: catalogs, kz / jscale / nmax_l per catalog, items and reductions per level ----
        std::vector<char> host;  // packed plan
        auto put = [&host](const void *p, size_t b) {
            const size_t o = al256(host.size());
            host.resize(o + b);
            memcpy(host.data() + o, p, b);
            return o;
        };
        std::vector<size_t> o_kz(gn), o_nl(gn), o_tm(gn);
        for (int c = c0; c < c1; ++c) {
            // TMA descriptors 0..3: the Legendre row sets (m pairs interleaved per point:
            // [lrp / 2][2 stride] FP32, 64 x 16 boxes = 32 m x 32 points); 4, 5, extended
            // range: the exponent sets by the parity of l ([tile][epitch] words, 128 x 1 boxes)
            CatPlan &P = cats[c];
            CUtensorMap tm[8];
            memset(tm, 0, sizeof(tm));
            char *rows = ws + off_rows[c - c0];
            const uint64_t lrp = (uint64_t)((P.in.lmax + 1) & ~1);
            const size_t set_bytes = (size_t)P.stride * lrp * sizeof(float);
            for (int k = 0; k < nsets; ++k)
                if (!tmap_2d(&tm[k], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, rows + k * set_bytes, 2 * (uint64_t)P.stride,
                             lrp / 2, 2 * (uint64_t)P.stride * sizeof(float), 2 * KT, 16)) {
                    set_error("cuTensorMapEncodeTiled failed for the Legendre rows");
                    return CATANA_ERR_CUDA;
                }
            if (ext) {
                const int ep = (P.in.lmax + 1) & ~1;
                char *ex = ws + off_exp[c - c0];
                for (int k = 0; k < 2; ++k)
                    if (!tmap_2d(&tm[4 + k], CU_TENSOR_MAP_DATA_TYPE_UINT64, ex + (size_t)k * exp_set_words(P) * 8,
                                 (uint64_t)ep, (uint64_t)P.ntiles, (uint64_t)ep * 8, 128, 1)) {
                        set_error("cuTensorMapEncodeTiled failed for the row exponents");
                        return CATANA_ERR_CUDA;
                    }
            }
            o_tm[c - c0] = put(tm, sizeof(tm));
        }
        for (int c = c0; c < c1; ++c) {
            CatPlan &P = cats[c];
            const int L = P.in.lmax, M = P.in.nmax;
            // J scale per (l, n): a power of two bringing max |w j_l(k_ln r)| over the
            // catalog's radii into [2^14, 2^15) -- j_l rises monotonically up to its
            // first maximum, so below it the largest radius sets the bound.  Modes whose
            // arguments stay deep below l keep their J values normal in FP16.
            std::vector<float4> kz((size_t)L * M);
            const SplitCache &C = ctx->split_cache;
            for (int l = 0; l < L; ++l)
                for (int n = 0; n < M; ++n) {
                    const size_t t = (size_t)l * M + n;
                    float hi, lo;
                    split_ff(P.kh[t] / H, hi, lo);
                    const double zl = P.kh[t] * P.max_r;
                    double mj = C.maxj[l];
                    if (l > 0 && zl < C.zpeak[l]) mj = std::min(mj, std::fabs(sbessel_jl(l, zl)));
                    mj = std::max(mj, 1e-300);
                    const int e = std::max(-60, std::min(110, (int)std::floor(std::log2(32768.0 / (mj * P.max_w)))));
                    const double js = std::ldexp(1.0, e);
                    kz[t] = make_float4(hi, lo, (float)js, (float)(1.0 / (js * Y_SCALE)));
                }
            o_kz[c - c0] = put(kz.data(), kz.size() * sizeof(float4));
            o_nl[c - c0] = put(P.nmax_l.data(), P.nmax_l.size() * sizeof(int));
        }
        // FP64 coefficients of the sectoral step, -sqrt((2l+1)/(2l)) for l < lmax_g
        std::vector<double> asect(lmax_g + 1, 0.0);
        for (int l = 1; l < lmax_g; ++l) asect[l] = -std::sqrt((2.0 * l + 1.0) / (2.0 * l));
        const size_t o_as = put(asect.data(), asect.size() * sizeof(double));
        // catalog descriptors (fixed for the group)
        const size_t o_cats = al256(host.size());
        host.resize(o_cats + (size_t)gn * sizeof(SplitCat));
        const size_t o_dyn = al256(host.size());  // items and reductions follow
        for (int c = c0; c < c1; ++c) {
            CatPlan &P = cats[c];
            SplitCat sc;
            sc.pts = reinterpret_cast<const SplitPt *>(ws + off_pts[c - c0]);
            sc.rows = reinterpret_cast<float *>(ws + off_rows[c - c0]);
            sc.n = P.in.n;
            sc.stride = (int)P.stride;
            sc.lrows = P.in.lmax;
            sc.lrp = (P.in.lmax + 1) & ~1;
            sc.kzw = P.in.nmax;
            sc.epitch = (P.in.lmax + 1) & ~1;
            sc.rexp = ext ? reinterpret_cast<unsigned long long *>(ws + off_exp[c - c0]) : nullptr;
            sc.eset = ext ? exp_set_words(P) : 0;
            sc.tmaps = nullptr;  // patched at upload
            sc.kz = nullptr;  // patched below, once the plan buffer's address is known
            sc.nmax_l = nullptr;
            memcpy(host.data() + o_cats + (size_t)(c - c0) * sizeof(SplitCat), &sc, sizeof(SplitCat));
        }
        // Work items of every level for a schedule of `waves` CTAs per SM and m-blocks of at
        // most `mcap` complex m (the MMA's N = 2 mcount): at level l the group's tiles x
        // m-blocks are cut into slabs of T tiles, T chosen so the items fill about waves x SMs
        // CTAs.  Items of one catalog are block-major.
        struct Sched {
            std::vector<SplitItem> items;
            std::vector<SplitRed> reds;
            std::vector<int> item0, red0, maxn;
            std::vector<char> fullj;  // per level: every item has 128 radial orders in its half
            std::vector<double> flops;
        };
        auto schedule = [&](double waves, int mcap, Sched &S) {
            S.items.clear();
            S.reds.clear();
            S.item0.assign(lmax_g + 1, 0);
            S.red0.assign(lmax_g + 1, 0);
            S.maxn.assign(lmax_g, 0);
            S.fullj.assign(lmax_g, 1);
            S.flops.assign(lmax_g, 0.0);
            for (int l = 0; l < lmax_g; ++l) {
                S.item0[l] = (int)S.items.size();
                S.red0[l] = (int)S.reds.size();
                const int nblocks = (l + 1 + mcap - 1) / mcap;
                const int mblk = (((l + 1 + nblocks - 1) / nblocks) + 3) & ~3;  // balanced, multiple of 4
                // the active catalogs, largest first: the CTAs of a launch start
                // roughly in index order, so the long items start first
                std::vector<int> act;
                int64_t tmax = 1;
                for (int c = c0; c < c1; ++c)
                    if (l < cats[c].in.lmax && cats[c].nmax_l[l] > 0) {
                        act.push_back(c);
                        tmax = std::max(tmax, cats[c].ntiles);
                    }
                std::stable_sort(act.begin(), act.end(),
                                 [&](int x, int y) { return cats[x].ntiles > cats[y].ntiles; });
                // slab length T: the largest for which the level still has at least
                // waves x SMs items (small catalogs contribute one short item each)
                const double slots = std::max(1.0, waves * ctx->sm_count);
                auto nitems = [&](int64_t T) {
                    double k = 0.0;
                    for (int c : act)
                        k += (double)nblocks * ((cats[c].nmax_l[l] + NHALF - 1) / NHALF) *
                             (double)((cats[c].ntiles + T - 1) / T);
                    return k;
                };
                int64_t T = 1;
                if (nitems(1) > slots) {
                    int64_t lo = 1, hi = tmax;  // nitems(lo) >= slots
                    while (lo < hi) {
                        const int64_t mid = lo + (hi - lo + 1) / 2;
                        if (nitems(mid) >= slots) lo = mid; else hi = mid - 1;
                    }
                    T = lo;
                }
                for (int c : act) {
                    CatPlan &P = cats[c];
                    const int nslabs = (int)((P.ntiles + T - 1) / T);
                    const int64_t Tc = (P.ntiles + nslabs - 1) / nslabs;  // even slabs within the catalog
                    SplitRed r;
                    r.item0 = (int)(S.items.size() - S.item0[l]);
                    r.nslabs = nslabs;
                    r.mblk = mblk;
                    r.nmax_l = P.nmax_l[l];
                    r.kzw = P.in.nmax;
                    r.nhalves = (P.nmax_l[l] + NHALF - 1) / NHALF;
                    r.fl = reinterpret_cast<double2 *>(P.in.f_acc) + (size_t)P.in.nmax * l * (l + 1) / 2;
                    r.kln_row = P.in.kln_dev + (size_t)l * P.in.nmax;
                    S.reds.push_back(r);
                    S.maxn[l] = std::max(S.maxn[l], P.nmax_l[l]);
                    S.flops[l] += 4.0 * (double)P.in.n * P.nmax_l[l] * (l + 1);
                    for (int bk = 0; bk < nblocks; ++bk) {
                        const int mb0 = bk * mblk;
                        for (int hf = 0; hf < r.nhalves; ++hf)
                            for (int sl = 0; sl < nslabs; ++sl) {
                                SplitItem it;
                                it.cat = c - c0;
                                it.mb0 = mb0;
                                it.mcount = std::min(mblk, l + 1 - mb0);
                                it.n0 = hf * NHALF;
                                if (std::min(NHALF, P.nmax_l[l] - it.n0) < NHALF) S.fullj[l] = 0;
                                it.t0 = (int64_t)sl * Tc;
                                it.t1 = std::min<int64_t>(P.ntiles, it.t0 + Tc);
                                S.items.push_back(it);
                            }
                    }
                }
            }
            S.item0[lmax_g] = (int)S.items.size();
            S.red0[lmax_g] = (int)S.reds.size();
        };
        // upload: [catalog tables | catalog descriptors | items | reductions]
        char *pd = nullptr;
        size_t o_items = 0, o_reds = 0;
        auto upload = [&](const Sched &S) -> catana_status_t {
            const size_t ib = S.items.size() * sizeof(SplitItem), rb = S.reds.size() * sizeof(SplitRed);
            o_items = o_dyn;
            o_reds = al256(o_items + ib);
            const size_t total = o_reds + rb + 256;
            CG_CUDA_TRY(ctx->split_plan.ensure(total));
            pd = ctx->split_plan.as<char>();
            host.resize(std::max(host.size(), total));
            for (int c = c0; c < c1; ++c) {
                SplitCat *sc = reinterpret_cast<SplitCat *>(host.data() + o_cats) + (c - c0);
                sc->kz = reinterpret_cast<const float4 *>(pd + o_kz[c - c0]);
                sc->tmaps = pd + o_tm[c - c0];
                sc->nmax_l = reinterpret_cast<const int *>(pd + o_nl[c - c0]);
            }
            if (ib) memcpy(host.data() + o_items, S.items.data(), ib);
            if (rb) memcpy(host.data() + o_reds, S.reds.data(), rb);
            CG_CUDA_TRY(cudaMemcpyAsync(pd, host.data(), o_reds + rb, cudaMemcpyHostToDevice, st));
            int max_items = 1;
            for (int l = 0; l < lmax_g; ++l) max_items = std::max(max_items, S.item0[l + 1] - S.item0[l]);
            CG_CUDA_TRY(ctx->partial.ensure((size_t)max_items * 256 * 128 * sizeof(float)));
            return CATANA_OK;
        };
        auto level_args = [&](const Sched &S, int l) {
            SplitArgs a;
            a.l = l;
            a.nint = nint;  // intervals this run reaches (the cached table may hold more; its row stride is nint_tab)
            a.items = reinterpret_cast<const SplitItem *>(pd + o_items) + S.item0[l];
            a.cats = reinterpret_cast<const SplitCat *>(pd + o_cats);
            a.coef = coef_d + (size_t)l * (l + 1) / 2;
            a.rcoef = coef_d + (size_t)lmax_tab * (lmax_tab + 1) / 2 + (size_t)l * (l + 1) / 2;
            a.tab = tab + (size_t)l * nint_tab * 2;
            a.partial = ctx->partial.as<float>();
            a.err = err_dev;
            a.wait_ns = stall_ns ? stall_ns : WAIT_NS;
            a.stall = stall_ns ? 1 : 0;
            return a;
        };

        double waves_use = waves;
        int mblk_use = mblk_cap;
        if (waves_use <= 0.0) {
            // autotune: time the contraction at three sample levels for each schedule
            // (the rows those launches write are rewritten by the real level loop)
            const std::string key = tune_key(cats, c0, c1);
            auto hit = ctx->split_tuned.find(key);
            if (hit != ctx->split_tuned.end()) {
                waves_use = hit->second.first;
                mblk_use = hit->second.second;
            } else {
                // the schedule (CTAs per SM) and the tile shape (m-block width: the MMA's N)
                const double cand[] = {1.0, 2.0, 3.0, 4.0, 6.0, 8.0, 12.0};
                const int mcand[] = {MBLK, 64};
                const int ls[3] = {std::max(1, lmax_g / 4), std::max(1, lmax_g / 2), std::max(1, (3 * lmax_g) / 4)};
                cudaEvent_t e0, e1;
                CG_CUDA_TRY(cudaEventCreate(&e0));
                CG_CUDA_TRY(cudaEventCreate(&e1));
                double best = 1e300;
                waves_use = 1.0;
                mblk_use = MBLK;
                Sched S;
                for (int rep = 0; rep < 2; ++rep)
                    for (int mc : mcand)
                    for (double w : cand) {
                        schedule(w, mc, S);
                        s = upload(S);
                        if (s != CATANA_OK) return s;
                        CG_CUDA_TRY(cudaEventRecord(e0, st));
                        for (int l : ls) {
                            if (l >= lmax_g) continue;
                            const int ni = S.item0[l + 1] - S.item0[l];
                            if (ni == 0) continue;
                            kern_for(S.fullj[l] != 0)<<<ni, NTOT, smem, st>>>(level_args(S, l));
                            count_launch();
                        }
                        CG_CUDA_TRY(cudaGetLastError());
                        CG_CUDA_TRY(cudaEventRecord(e1, st));
                        CG_CUDA_TRY(cudaEventSynchronize(e1));
                        float ms = 0.f;
                        CG_CUDA_TRY(cudaEventElapsedTime(&ms, e0, e1));
                        if (rep == 1 && ms < best) {
                            best = ms;
                            waves_use = w;
                            mblk_use = mc;
                        }
                    }
                cudaEventDestroy(e0);
                cudaEventDestroy(e1);
                ctx->split_tuned[key] = std::make_pair(waves_use, mblk_use);
            }
        }
        ctx->split_last_waves = waves_use;
        ctx->split_last_mblk = mblk_use;
        Sched S;
        schedule(waves_use, mblk_use, S);
        s = upload(S);
        if (s != CATANA_OK) return s;
        float *partial = ctx->partial.as<float>();
        // ---- FP64 sectoral seeds of every level, after the autotuner's trial launches
        // (which write rows) and before the level loop ----
        {
            for (int c = c0; c < c1; ++c) {
                const int64_t nt = cats[c].ntiles;
                if (cats[c].in.lmax < 2 || nt == 0) continue;
                k_split_sectoral<<<ceil_div(nt, 8), 256, 0, st>>>(reinterpret_cast<const SplitCat *>(pd + o_cats),
                                                                  c - c0, cats[c].in.lmax,
                                                                  reinterpret_cast<const double *>(pd + o_as), nt,
                                                                  (ext ? 2 : 0) | (rs ? 1 : 0));
                count_launch();
            }
            CG_CUDA_TRY(cudaGetLastError());
        }
        // ---- the level loop (optionally captured as one CUDA graph) ----
        auto levels = [&](bool profile, cudaStream_t ls_st) -> catana_status_t {
            for (int l = 0; l < lmax_g; ++l) {
                const int ni = S.item0[l + 1] - S.item0[l];
                const int nr = S.red0[l + 1] - S.red0[l];
                if (ni == 0) continue;
                if (profile) prof_begin(ls_st);
                kern_for(S.fullj[l] != 0)<<<ni, NTOT, smem, ls_st>>>(level_args(S, l));
                if (profile) prof_end(ls_st, S.flops[l]);
                dim3 rg(ceil_div((int64_t)(l + 1) * S.maxn[l], 128), nr);
                k_split_reduce<<<rg, 128, 0, ls_st>>>(partial, l + 1,
                                                   reinterpret_cast<const SplitRed *>(pd + o_reds) + S.red0[l]);
                count_launch(2);
                CG_CUDA_TRY(cudaGetLastError());
            }
            return CATANA_OK;
        };
        if (use_graph) {
            // captured on the context's own stream (the caller's may be the legacy
            // default stream, which cannot capture) and launched on the caller's
            if (!ctx->capture_stream)
                CG_CUDA_TRY(cudaStreamCreateWithFlags(&ctx->capture_stream, cudaStreamNonBlocking));
            cudaGraph_t graph = nullptr;
            CG_CUDA_TRY(cudaStreamBeginCapture(ctx->capture_stream, cudaStreamCaptureModeThreadLocal));
            catana_status_t ls = levels(false, ctx->capture_stream);
            cudaError_t ce = cudaStreamEndCapture(ctx->capture_stream, &graph);
            if (ls != CATANA_OK) {
                if (graph) cudaGraphDestroy(graph);
                return ls;
            }
            CG_CUDA_TRY(ce);
            cudaGraphExec_t exec = nullptr;
            cudaError_t ie = cudaGraphInstantiate(&exec, graph, 0);
            cudaGraphDestroy(graph);
            CG_CUDA_TRY(ie);
            cudaError_t le = cudaGraphLaunch(exec, st);
            cudaGraphExecDestroy(exec);
            CG_CUDA_TRY(le);
        } else {
            s = levels(true, st);
            if (s != CATANA_OK) return s;
        }
        // the next group reuses the workspace: stream order on `st` keeps them apart
    }
    CG_CUDA_TRY(cudaEventRecord(ctx->split_ws_event, st));
    return CATANA_OK;
}

catana_status_t split_raw_accumulate(DeviceContext *ctx, const double *points_dev, const double *weights_dev,
                                     int64_t npoints, int lmax, int nmax, double rmax, const double *kln_dev,
                                     double *f_acc_dev, int *err_dev, cudaStream_t st, bool accurate) {
    if (npoints == 0 || lmax == 0 || nmax == 0) return CATANA_OK;
    // chunks whose Legendre rows stay under 16 GB; they share the accumulator, so
    // split_run places each in its own group and runs the groups one after another
    const int64_t chunk = std::max<int64_t>(KT, std::min<int64_t>(npoints, (int64_t)(16e9 / (12.0 * lmax))));
    std::vector<SplitCatInput> v;
    for (int64_t c0 = 0; c0 < npoints; c0 += chunk) {
        SplitCatInput in;
        in.pts = points_dev + 3 * c0;
        in.w = weights_dev ? weights_dev + c0 : nullptr;
        in.n = std::min(chunk, npoints - c0);
        in.lmax = lmax;
        in.nmax = nmax;
        in.rmax = rmax;
        in.kmax = 0.0;
        in.kln_dev = const_cast<double *>(kln_dev);
        in.f_acc = f_acc_dev;
        in.accurate = accurate;
        v.push_back(in);
    }
    return split_run(ctx, v, false, 1.0, MBLK, err_dev, st);
}

}  // namespace catana_gpu

extern "C" catana_status_t catana_gpu_test_split_stall(uint32_t wait_us) {
    if (wait_us == 0 || wait_us > 1000000u) {
        catana_gpu::set_error("test_split_stall: wait_us must be in [1, 1000000]");
        return CATANA_ERR_ARG;
    }
    catana_gpu::g_split_stall_ns.store((uint64_t)wait_us * 1000ull);
    return CATANA_OK;
}
