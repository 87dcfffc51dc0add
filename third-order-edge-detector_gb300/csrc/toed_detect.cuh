// toed_detect.cuh -- fused single-pass TOED detection kernel (sm_103a).
//
// One persistent CTA (256 threads) repeatedly takes a work unit from an
// atomic queue.  A unit is a vertical strip of one image: 30 output columns
// (32 with a one-pixel ring) by S output rows.  The CTA slides down the strip
// in steps of B = 16 rows, keeping everything on chip:
//
//   1. B new input rows (+ halo) arrive by TMA, by per-thread async copies
//      (float32; the ASYNC instantiation) or by plain loads, and are
//      converted to FP32 into a ring of input rows;
//   2. row pass: twelve horizontal responses -- G, Gx, Gxx and Gxxx, each
//      truncated to 2r+1 taps (T), full 2r+3 taps (F) and half-pixel shifted
//      (S) -- into a ring of row-pass rows (G, Gx feed the dense first
//      derivatives, Gxx, Gxxx the per-edgel ones);
//   3. column pass: Ix and Iy at the four half-pixel sub-grids (the 2x grid
//      of the reference, cpu_toed.cpp:204-355) for the B new rows, and the
//      threshold test on |grad I|^2 as one ballot mask per (2x row, column
//      parity);
//   4. the points above the threshold listed in row-major order; subpixel
//      NMS along the gradient with the reference's 8-sector interpolation,
//      max test and parabola fit (cpu_toed.cpp:399-495), decided in FP32;
//      survivors compacted in order;
//   5. per edgel only: the seven higher derivatives, contracted from the
//      row-pass ring with the y taps of the edgel's sub-grid, then the
//      third-order orientation (cpu_toed.cpp:227-232) and the peak fit, its
//      cancelling sums taken on exact differences (HYBRID) or plain FP32;
//      records are deferred in a ring and finished by all threads at once;
//      the staged record goes to a staging area and the row's {offset,
//      count} to the row-segment table that the ordering pass
//      (toed_finalize.cu) turns into the reference's row-major edgel list.
//
// Both rings hold a multiple of 8 rows (the live window rounded up) and are
// indexed by absolute row, so sliding the window moves no data.
//
// Compared with the reference kernel (direct 17x17 and 19x19 sums of nine
// derivatives at every point, gpu_convolve.cu:114-131) this evaluates the
// separable form, keeps the nine-derivative stack off HBM entirely and
// computes seven of the nine derivatives only where an edgel survives.
#pragma once
#include "toed_common.cuh"

namespace toed {

__host__ __device__ constexpr size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

// NMS-window rows are kFxyStride float2 apart (FW = 2 kExt used): the two
// spare entries shift each row by four banks, so that the NMS stage's reads
// at scattered (row, column) points collide less.
constexpr int kFxyStride = 2 * kExt + 2;

template <int R>
struct Cfg {
    static constexpr int B = kStepRows;
    static constexpr int NT = 2 * R + 3;            // taps of a full / shifted filter
    static constexpr int NIN = kExt + 2 * R + 2;    // input columns held per row
    static constexpr int HS = B + 2 * R + 3;        // live rows of the row-pass window
    // ring rows (input and row-pass rings): HS rounded up to a multiple of 8,
    // so that ring row of slot 0 (advancing by B) stays a multiple of 8 and
    // the column pass knows where its window can wrap (col_pass)
    static constexpr int RING = (HS + 7) / 8 * 8;
    static constexpr int MS = 2 * B + 2;            // 2x-grid rows held for NMS
    static constexpr int NMS_ROWS = 2 * B;          // 2x-grid rows decided per step
    static constexpr int MAXC = NMS_ROWS * 2 * kInner;
    static constexpr int RECW = 21;                 // words per deferred edgel record (odd: no bank conflicts)
    static constexpr int FW = 2 * kExt;             // 2x-grid columns held per row
    // one TMA box of input rows, or two boxes of float32 rows for the async copies
    static constexpr size_t sz_raw = 2 * kStepRows * kRawRowBytes;
    static constexpr size_t off_raw = 0;
    static constexpr size_t off_mbar = off_raw + sz_raw;
    static constexpr size_t off_in = align_up(off_mbar + 16, 16);
    static constexpr size_t off_P = align_up(off_in + sizeof(float) * RING * NIN, 16);
    // row-pass ring rows are PS float2 apart: two spare entries per row shift
    // each row by four banks, so that the per-edgel stage's scattered reads
    // (one edgel's column per lane) collide less
    static constexpr int PS = kExt + 2;
    static constexpr size_t off_fxy = off_P + sizeof(float2) * 6 * RING * PS;
    static constexpr size_t off_mask = off_fxy + sizeof(float2) * MS * kFxyStride;
    static constexpr size_t off_list = off_mask + sizeof(unsigned) * MS * 2 * kHalves;
    static constexpr size_t off_tab = align_up(off_list + sizeof(unsigned) * MAXC, 16);
    static constexpr size_t off_misc = align_up(off_tab + sizeof(float4) * 3 * NT, 16);
    static constexpr size_t off_rec = off_misc + sizeof(int) * 256;
    // deferred-edgel ring: as many records as keep two CTAs per SM (<= 112 KB each)
    static constexpr int MINB = 2;
    static constexpr size_t budget = 112 * 1024;
    static constexpr int NREC_FIT = off_rec < budget ? (int)((budget - off_rec) / (RECW * 4) / 32 * 32) : 0;
    static constexpr int NREC = NREC_FIT > 256 ? 256 : (NREC_FIT < 64 ? 64 : NREC_FIT);
    static constexpr size_t smem = off_rec + sizeof(float) * RECW * NREC;
};

__device__ __forceinline__ float sqrt_approx(float x)
{
    float y;
    asm("sqrt.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// Image pixel as FP32 with zero padding outside the image (cpu_toed.cpp:207-208).
__device__ __forceinline__ float fetch_px(const void* src, long long pitch, int H, int W, int dtype,
                                          int y, int x)
{
    if ((unsigned)y >= (unsigned)H || (unsigned)x >= (unsigned)W) return 0.f;
    const long long o = (long long)y * pitch + x;
    if (dtype == TOED_U8) return (float)__ldg((const unsigned char*)src + o);
    return __ldg((const float*)src + o);
}

// ---------------------------------------------------------------------------
// TMA staging of input rows (cp.async.bulk.tensor + mbarrier)
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_addr(const void* p)
{
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint32_t bar)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// Thread 0: one box of kStepRows rows at (x, y) of image map `tm` into `dst`.
__device__ __forceinline__ void tma_load_rows(const CUtensorMap* tm, uint32_t dst, uint32_t bar, int x, int y,
                                              uint32_t bytes)
{
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
            dst),
        "l"(reinterpret_cast<uint64_t>(tm)), "r"(x), "r"(y), "r"(bar)
        : "memory");
}

// Bounded wait for the mbarrier phase: gives up after ~2^20 polls (each poll
// may suspend briefly) instead of hanging the SM.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t phase)
{
    for (int i = 0; i < (1 << 20); ++i) {
        uint32_t ok;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
            : "=r"(ok)
            : "r"(bar), "r"(phase)
            : "memory");
        if (ok) return true;
    }
    return false;
}

// Per-thread asynchronous 4-byte copy global -> shared; src_bytes 0 writes
// zero (the reference's zero padding outside the image).
__device__ __forceinline__ void cp_async4(uint32_t dst, const void* src, int src_bytes)
{
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"(dst), "l"(src), "r"(src_bytes) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// Ring row of x for 0 <= x < 2 * N (every ring index the kernel forms).
template <int N>
__device__ __forceinline__ int ring_wrap(int x) { return x >= N ? x - N : x; }

// Input rows by per-thread async copies (float32 rows at any address, e.g.
// page-locked host memory read through its device mapping), two boxes of B
// rows ahead in a double buffer.  A box is B rows x BW columns starting at
// the 16-byte-aligned column xa <= xin; thread t owns 16-byte chunk t of
// every box: one 16-byte copy where the image allows it (aligned base and
// rows, chunk inside the image), else four 4-byte copies with zero fill
// outside the image.  Each thread converts the chunk it copied itself, so it
// waits for its own copies only (cp.async.wait_group 1: the newest box may
// still be in flight).  Boxes 0 .. Q0-1 are the first step's window, box
// Q0 - 1 + s the new rows of step s >= 1.  Only the ASYNC instantiation of
// the kernel carries this path.
template <int R>
struct AsyncBox {
    using C = Cfg<R>;
    static constexpr int B = C::B;
    static constexpr int BW = (C::NIN + 3 + 3) / 4 * 4;          // box width (floats): NIN + the alignment shift
    static constexpr int CH = BW / 4;                           // 16-byte chunks per row
    static constexpr int Q0 = (C::HS + B - 1) / B;              // boxes of the first step
    static_assert(B * CH <= kThreads, "one chunk per thread");
    static_assert(2 * B * BW * 4 <= C::sz_raw, "two boxes fit the staging buffer");
};

// A thread's part of the async row staging, fixed for a work unit: its
// 16-byte chunk of every box (box row rr, chunk k: image columns x .. x+3,
// x = xa + 4k with xa the 16-byte-aligned column at or before the window's
// first column) and where the chunk's four floats go in the input ring.
struct AsyncLane {
    long long x;        // image column of the chunk's first float (may be < 0 at the left edge)
    int box;            // rr * BW + 4k: the chunk's offset in a box
    int ccol;           // 4k - shift: ring column of the chunk's first float
    int rr;             // box row
    unsigned cmask;     // bit e: ring column ccol + e lies in [0, NIN)
    unsigned imask;     // bit e: image column x + e lies in [0, W)
    bool full;          // one 16-byte copy: aligned rows and all four columns inside the image
    bool on;            // the thread owns a chunk (t < B * CH)
};

template <int R>
__device__ __forceinline__ AsyncLane async_lane(const float* fsrc, long long pitch, int W, int xin)
{
    using C = Cfg<R>;
    using A = AsyncBox<R>;
    AsyncLane l;
    const int t = threadIdx.x;
    l.on = t < A::B * A::CH;
    l.rr = t / A::CH;
    const int k = t - l.rr * A::CH;
    const int xa = xin - (((xin % 4) + 4) % 4), shift = xin - xa;
    l.x = xa + 4 * k;
    l.box = l.rr * A::BW + 4 * k;
    l.ccol = 4 * k - shift;
    l.cmask = 0u;
    l.imask = 0u;
#pragma unroll
    for (int e = 0; e < 4; ++e) {
        if (l.ccol + e >= 0 && l.ccol + e < C::NIN) l.cmask |= 1u << e;
        if ((unsigned long long)(l.x + e) < (unsigned long long)W) l.imask |= 1u << e;
    }
    const bool al16 = ((reinterpret_cast<uintptr_t>(fsrc) & 15u) == 0) && ((pitch & 3) == 0);
    l.full = al16 && l.imask == 0xFu;
    return l;
}

template <int R>
__device__ __forceinline__ void async_issue_box(float* rawf, const float* fsrc, long long pitch, int H,
                                                const AsyncLane& l, int ys, int nsteps, int q)
{
    using A = AsyncBox<R>;
    constexpr int B = A::B;
    const int last = A::Q0 + nsteps - 2;  // the last box of the unit
    if (q <= last && l.on) {
        const int row0 = (q < A::Q0) ? ys - R - 3 + q * B : ys + (q - A::Q0 + 1) * B + R;
        const int y = row0 + l.rr;
        float* dst = rawf + (q & 1) * (B * A::BW) + l.box;
        const bool rowin = (unsigned)y < (unsigned)H;
        const float* srow = fsrc + (rowin ? (long long)y * pitch + l.x : 0);
        if (l.full) {
            // rows outside the image: zero fill, nothing read
            asm volatile("cp.async.ca.shared.global [%0], [%1], 16, %2;" ::"r"(smem_addr(dst)), "l"(srow),
                         "r"(rowin ? 16 : 0)
                         : "memory");
        } else {
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                const bool in = rowin && ((l.imask >> e) & 1u);
                cp_async4(smem_addr(dst + e), in ? srow + e : fsrc, in ? 4 : 0);
            }
        }
    }
    cp_async_commit();  // one group per box, empty past the last box, so that wait_group counts boxes
}

template <int R>
__device__ __forceinline__ void stage_rows_async(float* __restrict__ sIn, unsigned char* sRaw, const float* fsrc,
                                                 long long pitch, int H, const AsyncLane& l, int ys, int s,
                                                 int nsteps, int rb, int* dbg)
{
    using C = Cfg<R>;
    using A = AsyncBox<R>;
    constexpr int B = C::B;
    float* rawf = reinterpret_cast<float*>(sRaw);
    if (s == 0) {
        async_issue_box<R>(rawf, fsrc, pitch, H, l, ys, nsteps, 0);
        async_issue_box<R>(rawf, fsrc, pitch, H, l, ys, nsteps, 1);
    }
    const int q0 = (s == 0) ? 0 : A::Q0 - 1 + s, q1 = (s == 0) ? A::Q0 : q0 + 1;
    for (int q = q0; q < q1; ++q) {
        asm volatile("cp.async.wait_group 1;" ::: "memory");
        const int nrows = (s == 0) ? min(B, C::HS - q * B) : B;
        const int a0 = (s == 0) ? q * B : rb + 2 * R + 3;  // ring row of the box's row 0 (before wrapping)
        if (l.on && l.rr < nrows) {
            const float4 v = *reinterpret_cast<const float4*>(rawf + (q & 1) * (B * A::BW) + l.box);
            const int ph = ring_wrap<C::RING>(a0 + l.rr);
            float* dst = sIn + ph * C::NIN + l.ccol;
            if (TOED_IN_BOUNDS(ph < C::RING && (q & 1) * (B * A::BW) + l.box + 3 < 2 * B * A::BW, dbg)) {
                if (l.cmask & 1u) dst[0] = v.x;
                if (l.cmask & 2u) dst[1] = v.y;
                if (l.cmask & 4u) dst[2] = v.z;
                if (l.cmask & 8u) dst[3] = v.w;
            }
        }
        async_issue_box<R>(rawf, fsrc, pitch, H, l, ys, nsteps, q + 2);
    }
}

// ---------------------------------------------------------------------------
// Row pass: for ring rows p0, p0+1, ... (mod RING; nrows of them) of the
// input ring write the same rows of the row-pass ring.  Item = (row, pair of ext columns 2k, 2k+1).
// Planes: 0 PT=(T_G,T_Gx) 1 PF=(F_G,F_Gx) 2 PS=(S_G,S_Gx)
//         3 QT=(T_Gxx,T_Gxxx) 4 QF 5 QS, each [RING][PS] float2 (32 used per row).
// Convolution direction as the reference: out(x) = sum_q in(x-q) X(q).
// ---------------------------------------------------------------------------
template <int R>
__device__ __forceinline__ void row_pass(const float* __restrict__ sIn, int p0, int nrows,
                                         float2* __restrict__ sP, const TapBlock& tp, int* dbg)
{
    using C = Cfg<R>;
    constexpr int NV = 2 * R + 4;
    for (int item = threadIdx.x; item < nrows * (kExt / 2); item += kThreads) {
        const int i = item / (kExt / 2), k = item % (kExt / 2);
        const int ph = ring_wrap<C::RING>(p0 + i);
        if (!TOED_IN_BOUNDS(ph < C::RING && 2 * k + NV <= C::NIN, dbg)) continue;
        const float2* src = reinterpret_cast<const float2*>(sIn + ph * C::NIN + 2 * k);
        float v[NV];
#pragma unroll
        for (int t = 0; t < NV / 2; ++t) {
            const float2 q = src[t];
            v[2 * t] = q.x;
            v[2 * t + 1] = q.y;
        }
        float o_[2][12];
#pragma unroll
        for (int o = 0; o < 2; ++o) {
            // The odd filters (Gx, Gxxx) are exactly antisymmetric about 0 (about
            // -1/2 for the shifted set): each mirrored pair of inputs is
            // differenced once -- fewer operations and a smaller rounding
            // error, since neighbouring inputs nearly cancel.  The even filters
            // (G, Gxx) are summed tap by tap: folding them would round the sum
            // of two full-scale inputs and double the error of Gxx.
            const int c = o + R + 1;  // centre: out(x) = sum_q in(x-q) X(q), in(x-q) = v[c-q]
            float tG = 0.f, tGxx = 0.f, tGx = 0.f, tGxxx = 0.f;
#pragma unroll
            for (int q = -R; q <= R; ++q) {
                tG = fmaf(v[c - q], tp.v[0][q + R + 1], tG);
                tGxx = fmaf(v[c - q], tp.v[2][q + R + 1], tGxx);
            }
#pragma unroll
            for (int q = 1; q <= R; ++q) {
                const float df = v[c - q] - v[c + q];
                tGx = fmaf(df, tp.v[1][q + R + 1], tGx);
                tGxxx = fmaf(df, tp.v[3][q + R + 1], tGxxx);
            }
            // full 2r+3-tap responses add the taps q = +-(r+1)
            const float fG = fmaf(v[c + R + 1], tp.v[0][0], fmaf(v[c - R - 1], tp.v[0][2 * R + 2], tG));
            const float fGxx = fmaf(v[c + R + 1], tp.v[2][0], fmaf(v[c - R - 1], tp.v[2][2 * R + 2], tGxx));
            const float dfo = v[c - R - 1] - v[c + R + 1];
            const float fGx = fmaf(dfo, tp.v[1][2 * R + 2], tGx);
            const float fGxxx = fmaf(dfo, tp.v[3][2 * R + 2], tGxxx);
            // shifted taps X(q + 1/2), q = -(r+1)..r+1: even filters tap by tap,
            // odd ones over the pairs (q, -1-q) for q = 0..r plus q = r+1 alone
            float sG = 0.f, sGxx = 0.f;
#pragma unroll
            for (int q = -(R + 1); q <= R + 1; ++q) {
                sG = fmaf(v[c - q], tp.v[4][q + R + 1], sG);
                sGxx = fmaf(v[c - q], tp.v[6][q + R + 1], sGxx);
            }
            const float vl = v[c - R - 1];
            float sGx = vl * tp.v[5][2 * R + 2], sGxxx = vl * tp.v[7][2 * R + 2];
#pragma unroll
            for (int q = 0; q <= R; ++q) {
                const float df = v[c - q] - v[c + 1 + q];
                sGx = fmaf(df, tp.v[5][q + R + 1], sGx);
                sGxxx = fmaf(df, tp.v[7][q + R + 1], sGxxx);
            }
            o_[o][0] = tG;  o_[o][1] = tGx;  o_[o][2] = fG;  o_[o][3] = fGx;
            o_[o][4] = sG;  o_[o][5] = sGx;  o_[o][6] = tGxx; o_[o][7] = tGxxx;
            o_[o][8] = fGxx; o_[o][9] = fGxxx; o_[o][10] = sGxx; o_[o][11] = sGxxx;
        }
#pragma unroll
        for (int a = 0; a < 6; ++a) {
            float4* dst = reinterpret_cast<float4*>(sP + (a * C::RING + ph) * C::PS + 2 * k);
            *dst = make_float4(o_[0][2 * a], o_[0][2 * a + 1], o_[1][2 * a], o_[1][2 * a + 1]);
        }
    }
}

// ---------------------------------------------------------------------------
// Column pass for one (column, sub-grid, 8-row group): Ix and Iy.  Window
// rows are read from the row-pass ring: logical slot h <-> ring row
// (rb + h) mod RING, rb the ring row of slot 0 at this step.
// V = 0: unshifted y taps truncated to 2r+1 (sub-grid (0,0), cpu_toed.cpp:205-221)
// V = 1: unshifted y taps, full 2r+3 (sub-grid (0,1/2), :246-262)
// V = 2: shifted y taps (sub-grids (1/2, .), :287-344)
// ---------------------------------------------------------------------------
template <int R, int V>
__device__ __forceinline__ void col_pass(const float2* __restrict__ P, int rb, int g, int col,
                                         const TapBlock& tp, float (&fx)[kColRows],
                                         float (&fy)[kColRows])
{
    using C = Cfg<R>;
    constexpr int YF = (V == 2) ? 4 : 0;
    constexpr int NW = kColRows + 2 * R + 2;  // window rows
    // Window row t is ring row (r0 + t) mod RING.  RING, rb and 8g are
    // multiples of 8, so r0 = 1 (mod 8) and the wrap, if any, falls at
    // t = 7 (mod 8): every block of window rows t in [8b - 1, 8b + 7) reads
    // from one base pointer, chosen once, plus a constant offset.
    static_assert(C::RING % 8 == 0 && kStepRows % 8 == 0 && kColRows == 8, "column-pass wrap blocks");
    constexpr int NBLK = (NW + 8) / 8;
#pragma unroll
    for (int o = 0; o < kColRows; ++o) { fx[o] = 0.f; fy[o] = 0.f; }
    const int r0 = ring_wrap<C::RING>(rb + g * kColRows + 1);
    const int tw = C::RING - r0;  // first window row past the ring's end
    const float2* base[NBLK];
#pragma unroll
    for (int b = 0; b < NBLK; ++b)
        base[b] = P + (r0 - ((8 * b - 1 >= tw) ? C::RING : 0)) * C::PS + col;
#pragma unroll
    for (int t = 0; t < NW; ++t) {
        const float2 h = base[(t + 1) / 8][t * C::PS];
#pragma unroll
        for (int o = 0; o < kColRows; ++o) {
            const int p = o + R + 1 - t;
            const bool in = (V == 0) ? (p >= -R && p <= R) : (p >= -(R + 1) && p <= R + 1);
            if (in) {
                fx[o] = fmaf(h.y, tp.v[YF + 0][p + R + 1], fx[o]);
                fy[o] = fmaf(h.x, tp.v[YF + 1][p + R + 1], fy[o]);
            }
        }
    }
}

// |grad I| at a 2x-grid point from its (Ix, Iy); the column pass, the NMS
// decision and the per-edgel epilogue all use this one expression.
__device__ __forceinline__ float grad_mag(float2 g) { return sqrt_approx(fmaf(g.x, g.x, g.y * g.y)); }

// NMS evaluation at 2x-grid slot (m, c) of the step window.  Shared by the
// decision stage and the per-edgel epilogue so both see identical numbers.
struct NmsEval {
    float mv, gx, gy, nx, ny, slope, Map, Mdp, Mam, Mdm;
    bool cand;
};

// TOD (the corrected-normal mode, an extension beyond the reference): the
// sector, neighbours, fit and offset are taken along the unit vector of
// (tx, ty) -- the third-order vector -- instead of along (Ix, Iy); the
// candidate tests (threshold, gradient epsilon) stay those of the reference.
// The decision stage reads only `cand`; the unit normal (nx, ny) is formed
// for the per-edgel record and drops out of the decision code.
template <bool TOD = false>
__device__ __forceinline__ NmsEval nms_eval(const float2* __restrict__ sFxy, int m, int c, float thr,
                                            float tx = 0.f, float ty = 0.f, int* dbg = nullptr)
{
    NmsEval r;
    r.cand = false;
    constexpr int FS = kFxyStride;
    const float2 g = sFxy[m * FS + c];
    r.mv = grad_mag(g);
    if (!(r.mv > thr)) return r;  // cpu_toed.cpp:403 (also rejects NaN)
    r.gx = g.x;
    r.gy = g.y;
    if (fabsf(g.x) < 10e-6f && fabsf(g.y) < 10e-6f) return r;  // :407
    float dx = g.x, dy = g.y;
    if (TOD) {
        const float tm = sqrtf(fmaf(tx, tx, ty * ty));
        if (!(tm > 0.f) || !isfinite(tm)) return r;  // no direction
        r.nx = tx / tm;
        r.ny = ty / tm;
        dx = tx;
        dy = ty;
    } else {
        r.nx = __fdividef(g.x, r.mv);
        r.ny = __fdividef(g.y, r.mv);
    }
    // Eight sectors of cpu_toed.cpp:415-462 in closed form: x-major when
    // |Ix| >= |Iy|; the axis neighbour steps along the major axis towards
    // the gradient, the diagonal one along both; fm mirrors fp.  The slope
    // (minor over major component of the unit normal) is the ratio of the
    // direction's own components, the normalisation cancelling.
    const float ax = fabsf(dx), ay = fabsf(dy);
    const bool xmaj = ax >= ay;
    const int sx = (dx >= 0.f) ? 1 : -1, sy = (dy >= 0.f) ? 1 : -1;
    r.slope = __fdividef(fminf(ax, ay), fmaxf(ax, ay));
    const int ar = xmaj ? 0 : sy, ac = xmaj ? sx : 0;
#ifdef TOED_DEBUG_BOUNDS
    if (!TOED_IN_BOUNDS(m >= 1 && m + 1 < 2 * kStepRows + 2 && c >= 1 && c + 1 < 2 * kExt, dbg)) return r;
#endif
    r.Map = grad_mag(sFxy[(m + ar) * FS + c + ac]);
    r.Mdp = grad_mag(sFxy[(m + sy) * FS + c + sx]);
    r.Mam = grad_mag(sFxy[(m - ar) * FS + c - ac]);
    r.Mdm = grad_mag(sFxy[(m - sy) * FS + c - sx]);
    const float fp = r.Map * (1.f - r.slope) + r.Mdp * r.slope;
    const float fm = r.Mam * (1.f - r.slope) + r.Mdm * r.slope;
    const float mv = r.mv;
    const bool maxt = (mv > fm && mv >= fp) || (mv >= fm && mv > fp);  // :466-468
    // s* = -B/(2A) with A = (fm+fp-2f)/(2s^2), B = (fp-fm)/(2s), s = sqrt(1 +
    // slope^2) (:471-476), kept when |s*| <= sqrt(2) (:478), tested as
    // |fp - fm| s <= 2 sqrt(2) |fm + fp - 2f| without the division.  The max
    // test gives fm + fp <= 2f, so the denominator is negative unless it is
    // zero, where s* is inf or 0/0 and the point is rejected as before.
    const float num = fp - fm, den = fm + fp - 2.f * mv;
    r.cand = maxt && den < 0.f && fabsf(num) * sqrt_approx(fmaf(r.slope, r.slope, 1.f)) <= -2.82842712f * den;
    return r;
}

// The decision of nms_eval (gradient direction) without branches, for the
// NMS stage: every value is formed unconditionally (the neighbour offsets are
// within one row and column whatever the gradient) and the tests are combined
// at the end, so a warp runs it as one straight sequence.
__device__ __forceinline__ bool nms_decide(const float2* __restrict__ sFxy, int m, int c, float thr, int* dbg = nullptr)
{
    constexpr int FS = kFxyStride;
#ifdef TOED_DEBUG_BOUNDS
    if (!TOED_IN_BOUNDS(m >= 1 && m + 1 < 2 * kStepRows + 2 && c >= 1 && c + 1 < 2 * kExt, dbg)) return false;
#endif
    const float2 g = sFxy[m * FS + c];
    const float mv = grad_mag(g);
    const float ax = fabsf(g.x), ay = fabsf(g.y);
    const bool xmaj = ax >= ay;
    const int sx = (g.x >= 0.f) ? 1 : -1, sy = (g.y >= 0.f) ? 1 : -1;
    const float slope = __fdividef(fminf(ax, ay), fmaxf(ax, ay));
    const int ar = xmaj ? 0 : sy, ac = xmaj ? sx : 0;
    const float Map = grad_mag(sFxy[(m + ar) * FS + c + ac]);
    const float Mdp = grad_mag(sFxy[(m + sy) * FS + c + sx]);
    const float Mam = grad_mag(sFxy[(m - ar) * FS + c - ac]);
    const float Mdm = grad_mag(sFxy[(m - sy) * FS + c - sx]);
    const float fp = Map * (1.f - slope) + Mdp * slope;
    const float fm = Mam * (1.f - slope) + Mdm * slope;
    const bool maxt = (mv > fm && mv >= fp) || (mv >= fm && mv > fp);
    const float num = fp - fm, den = fm + fp - 2.f * mv;
    return (mv > thr) && !(ax < 10e-6f && ay < 10e-6f) && maxt && den < 0.f &&
           fabsf(num) * sqrt_approx(fmaf(slope, slope, 1.f)) <= -2.82842712f * den;
}

// The seven higher derivatives at 2x-grid slot (m, c) of the step window
// from the row-pass ring (the Q planes hold the Gxx / Gxxx row responses):
// fxx, fxy, fyy, fxxy, fxyy, fxxx, fyyy, contracted with the y taps of the
// point's sub-grid.  Used by the per-edgel stage and, in the corrected-normal
// mode, by the NMS decision, so that both see identical numbers.
template <int R>
__device__ __forceinline__ void gather_hi(const float2* __restrict__ sP, const float4* __restrict__ sTab, int rb, int m,
                                          int c, float (&d)[7], int* dbg = nullptr)
{
    using C = Cfg<R>;
    constexpr int NT = C::NT;
    const int a = m & 1, xe = c >> 1, b = c & 1;
    const int xv = b ? 2 : (a ? 1 : 0);
    const int yv = a ? 2 : (b ? 1 : 0);
    const float2* Pp = sP + xv * C::RING * C::PS + xe;
    const float2* Qp = sP + (3 + xv) * C::RING * C::PS + xe;
    const float4* tab = sTab + yv * NT;
    float fxy = 0.f, fyy = 0.f, fxyy = 0.f, fyyy = 0.f, fxx = 0.f, fxxy = 0.f, fxxx = 0.f;
    const int h0 = rb + (m >> 1);
#ifdef TOED_DEBUG_BOUNDS
    if (!TOED_IN_BOUNDS(xe >= 0 && xe < kExt && h0 >= 0 && h0 + NT - 1 < 2 * C::RING, dbg)) {
        for (int f = 0; f < 7; ++f) d[f] = 0.f;
        return;
    }
#endif
    // window row kk is ring row hw + kk, less RING from kk = tw on
    const int hw = ring_wrap<C::RING>(h0), tw = C::RING - hw;
    const float2* Pb = Pp + hw * C::PS;
    const float2* Qb = Qp + hw * C::PS;
#pragma unroll
    for (int kk = 0; kk < NT; ++kk) {
        const int ph = kk * C::PS - ((kk >= tw) ? C::RING * C::PS : 0);
        const float2 hp = Pb[ph];
        const float2 hq = Qb[ph];
        const float4 t = tab[NT - 1 - kk];
        fxy = fmaf(hp.y, t.y, fxy);
        fyy = fmaf(hp.x, t.z, fyy);
        fxyy = fmaf(hp.y, t.z, fxyy);
        fyyy = fmaf(hp.x, t.w, fyyy);
        fxx = fmaf(hq.x, t.x, fxx);
        fxxy = fmaf(hq.x, t.y, fxxy);
        fxxx = fmaf(hq.y, t.x, fxxx);
    }
    d[0] = fxx; d[1] = fxy; d[2] = fyy; d[3] = fxxy; d[4] = fxyy; d[5] = fxxx; d[6] = fyyy;
}

// The third-order vector (cpu_toed.cpp:227-230) in FP32 with its shared
// products factored out (the corrected-normal direction of the NMS).
__device__ __forceinline__ void to_vec32(float gx, float gy, const float (&d)[7], float* tix, float* tiy)
{
    const float fxx = d[0], fxy = d[1], fyy = d[2], fxxy = d[3], fxyy = d[4], fxxx = d[5], fyyy = d[6];
    const float a2 = fmaf(fxx, fxx, fxy * fxy), c2 = fmaf(fyy, fyy, fxy * fxy), bc = fxy * (fxx + fyy);
    const float pxy = gx * gy, x2 = gx * gx, y2 = gy * gy;
    *tix = fmaf(2.f, fmaf(gx, a2, fmaf(gy, bc, pxy * fxxy)), fmaf(y2, fxyy, x2 * fxxx));
    *tiy = fmaf(2.f, fmaf(gx, bc, fmaf(gy, c2, pxy * fxyy)), fmaf(x2, fxxy, y2 * fyyy));
}

// Per-edgel epilogue from a deferred record: peak fit (in HYB mode with the
// cancellations in fm + fp - 2f and fp - fm taken on exact differences) and the third-order
// orientation (cpu_toed.cpp:227-232; in HYB mode listed for the FP64
// recomputation when the vector nearly cancels), then the staged
// output record (x, y, orientation, strength) at its reserved slot.  The
// record holds its image's index; W2 is that image's 2x-grid width.
template <bool HYB>
__device__ __noinline__ void finish_edgel(const float* __restrict__ rc, const Scratch& sc, int W2)
{
    const float gx = rc[0], gy = rc[1], mv = rc[2], nx = rc[3], ny = rc[4], sl = rc[5];
    const float Map = rc[6], Mdp = rc[7], Mam = rc[8], Mdm = rc[9];
    const float fxx = rc[10], fxy = rc[11], fyy = rc[12], fxxy = rc[13], fxyy = rc[14], fxxx = rc[15],
                fyyy = rc[16];
    const int Gr = __float_as_int(rc[17]), Gc = __float_as_int(rc[18]);
    const int dst = __float_as_int(rc[19]), img = __float_as_int(rc[20]), idx = Gr * W2 + Gc;
    float x, y;  // the staged position (det_xy)
    float ori, str;
    if (HYB) {
        // fp - fm and fm + fp - 2f cancel.  With fp = Map + s (Mdp - Map) and
        // fm = Mam + s (Mdm - Mam) both are formed from differences of nearly
        // equal FP32 magnitudes (exact within a factor 2 of each other), the
        // interpolation weight applied last:
        //   fp - fm        = dA + s (dD - dA),  dA = Map - Mam, dD = Mdp - Mdm
        //   fm + fp - 2f   = eA + s (eD - eA),  eA = (Map - f) + (Mam - f), eD likewise
        // so no full-scale sum is rounded before the cancellation.
        const float dA = Map - Mam, dD = Mdp - Mdm;
        const float eA = (Map - mv) + (Mam - mv), eD = (Mdp - mv) + (Mdm - mv);
        const float num = fmaf(sl, dD - dA, dA);
        const float den = fmaf(sl, eD - eA, eA);
        const float ss = sqrtf(1.f + sl * sl);
        const float sst = -0.5f * num * ss / den;           // s* = -B / (2A)
        const float maxf = mv - 0.125f * num * num / den;   // A s*^2 + B s* + C
        // (pos - 1) / 2, cpu_toed.cpp:516: the grid coordinate is exact, the
        // subpixel offset is staged alone and added in FP64 when the list is
        // written, so that large coordinates keep it
        x = 0.5f * sst * nx;
        y = 0.5f * sst * ny;
        str = sqrtf((maxf * nx) * (maxf * nx) + (maxf * ny) * (maxf * ny));
        // cpu_toed.cpp:227-232 with the shared products factored out, in FP32:
        // TIx = 2 (fx (fxx^2 + fxy^2) + fy fxy (fxx + fyy) + fx fy fxxy) + fy^2 fxyy + fx^2 fxxx
        // TIy = 2 (fx fxy (fxx + fyy) + fy (fyy^2 + fxy^2) + fx fy fxyy) + fx^2 fxxy + fy^2 fyyy
        // Its own rounding reaches the angle times the cancellation ratio
        // below (~1e-7 x ratio); the ill-conditioned vectors are recomputed
        // in FP64 from FP64 derivatives, so FP64 here would buy nothing.
        const float a2 = fmaf(fxx, fxx, fxy * fxy), c2 = fmaf(fyy, fyy, fxy * fxy), bc = fxy * (fxx + fyy);
        const float pxy = gx * gy, x2 = gx * gx, y2 = gy * gy;
        const float tixf = fmaf(2.f, fmaf(gx, a2, fmaf(gy, bc, pxy * fxxy)), fmaf(y2, fxyy, x2 * fxxx));
        const float tiyf = fmaf(2.f, fmaf(gx, bc, fmaf(gy, c2, pxy * fxyy)), fmaf(x2, fxxy, y2 * fyyy));
        ori = (tixf == 0.f && tiyf == 0.f) ? __int_as_float(0x7fc00000) : atan2f(tixf, -tiyf);
        // Cancellation ratio of the third-order vector: the sum of its terms'
        // magnitudes over its own size.  The FP32 derivative stack's rounding
        // reaches the orientation multiplied by this ratio, so edgels above
        // kRefineKappa are listed for the FP64 recomputation (refine_edgels).
        const float ax = fabsf(gx), ay = fabsf(gy), pxx = fabsf(fxx * fxy), pyy = fabsf(fyy * fxy);
        const float sabs = 2.f * ax * (fxx * fxx + fxy * fxy) + 2.f * ay * (fyy * fyy + fxy * fxy) +
                           2.f * (ax + ay) * (pxx + pyy) + 2.f * ax * ay * (fabsf(fxxy) + fabsf(fxyy)) +
                           ay * ay * (fabsf(fxyy) + fabsf(fyyy)) + ax * ax * (fabsf(fxxx) + fabsf(fxxy));
        const float tmax = fmaxf(fabsf(tixf), fabsf(tiyf));
        if (sabs > kRefineKappa * tmax && sc.refine_cap > 0 && dst < sc.staging_cap) {
            const int slot = atomicAdd(&sc.words[3], 1);
            if (slot < sc.refine_cap) sc.refine[slot] = make_int4(dst, img, Gr, Gc);
        }
    } else {
        const float fp = Map * (1.f - sl) + Mdp * sl;
        const float fm = Mam * (1.f - sl) + Mdm * sl;
        const float num = fp - fm, den = fm + fp - 2.f * mv;
        const float ss = sqrtf(1.f + sl * sl);
        const float sst = -0.5f * num * ss / den;
        const float maxf = mv - 0.125f * num * num / den;
        x = (float)Gc + sst * nx;  // the FP32 position on the 2x grid
        y = (float)Gr + sst * ny;
        str = sqrtf((maxf * nx) * (maxf * nx) + (maxf * ny) * (maxf * ny));
        const float tix = gx * (2.f * fxx * fxx + 2.f * fxy * fxy) + gy * (2.f * fxx * fxy + 2.f * fyy * fxy) +
                          2.f * gx * gy * fxxy + gy * gy * fxyy + gx * gx * fxxx;
        const float tiy = gx * (2.f * fxx * fxy + 2.f * fyy * fxy) + gy * (2.f * fyy * fyy + 2.f * fxy * fxy) +
                          2.f * gx * gy * fxyy + gx * gx * fxxy + gy * gy * fyyy;
        ori = (tix == 0.f && tiy == 0.f) ? __int_as_float(0x7fc00000) : atan2f(tix, -tiy);
    }
    if (dst < sc.staging_cap) {
        det_stage(sc)[dst] = make_float4(x, y, ori, str);
        sc.staging_idx[dst] = idx;
    }
}

// Bounded wait (one thread) until a copy group's ready flag reads `epoch`:
// the copy engine writes the flag after the group's pixels, in stream order.
// Returns false -- the unit is skipped -- once `spins` polls have gone by, or
// while the flag is not yet set and some CTA's wait has already given up
// (TOED_FLAG_TIMEOUT in words[2], checked after the first poll and every 256
// polls): a lost copy costs one bounded wait per resident CTA, not one per
// work unit, and units whose group did arrive are still detected.
static __device__ __noinline__ bool wait_ready(const int* flag, int epoch, int spins, int* words)
{
    for (int it = 0; it < spins; ++it) {
        int v;
        asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(flag) : "memory");
        if (v == epoch) return true;
        if ((it & 255) == 0) {
            int f;
            asm volatile("ld.relaxed.gpu.global.b32 %0, [%1];" : "=r"(f) : "l"(words + 2) : "memory");
            if (f & TOED_FLAG_TIMEOUT) return false;
        }
        __nanosleep(256);
    }
    atomicOr(&words[2], TOED_FLAG_TIMEOUT);
    return false;
}

// ASYNC: input rows by per-thread async copies (images with tma == 2) or
// plain loads; otherwise by TMA (tma == 1) or plain loads.  NMSTO: NMS and
// peak fit along the corrected normal (TOED_NMS_TO_NORMAL).
template <int R, bool HYB, bool ASYNC, bool NMSTO = false>
__global__ void __launch_bounds__(kThreads, Cfg<R>::MINB) toed_detect_kernel(const __grid_constant__ BatchParams p)
{
    using C = Cfg<R>;
    constexpr int B = C::B;
    constexpr int NT = C::NT;
    static_assert(kThreads / 32 == 8 * kHalves, "column pass: one warp per (sub-grid, 8-row group, half)");
    static_assert(2 * B == 32, "row scans: one lane per NMS row");
    extern __shared__ __align__(16) unsigned char smem[];
    float* sIn = reinterpret_cast<float*>(smem + C::off_in);
    float2* sP = reinterpret_cast<float2*>(smem + C::off_P);
    float2* sFxy = reinterpret_cast<float2*>(smem + C::off_fxy);
    unsigned* sMask = reinterpret_cast<unsigned*>(smem + C::off_mask);  // [MS][2] threshold ballots
    unsigned* sList = reinterpret_cast<unsigned*>(smem + C::off_list);
    float4* sTab = reinterpret_cast<float4*>(smem + C::off_tab);
    int* sMisc = reinterpret_cast<int*>(smem + C::off_misc);
    float* sRec = reinterpret_cast<float*>(smem + C::off_rec);
    int* sAccCnt = sMisc + 64;   // [32] accepted edgels per NMS row
    int* sWarp = sMisc + 96;     // [2][16] warp counts of the NMS compaction
    int* sScal = sMisc + 128;    // [0] unit [1] staging refill
    unsigned char* sRaw = smem + C::off_raw;  // TMA destination: one box of input rows
    const uint32_t bar = smem_addr(smem + C::off_mbar);
    uint32_t phase = 0;

    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const TapBlock& tp = p.taps;

    // y-direction tap table for the per-edgel stage: [variant][k] = (G, Gy, Gyy, Gyyy)
    for (int i = tid; i < 3 * NT; i += kThreads) {
        const int v = i / NT, k = i % NT;
        const int f = (v == 2) ? 4 : 0;
        float4 t = make_float4(tp.v[f][k], tp.v[f + 1][k], tp.v[f + 2][k], tp.v[f + 3][k]);
        if (v == 0 && (k == 0 || k == NT - 1)) t = make_float4(0.f, 0.f, 0.f, 0.f);
        sTab[i] = t;
    }
    int nrec = 0;  // deferred records in the ring (uniform across the CTA)
    int stg_next = 0, stg_end = 0;  // this CTA's reserved staging range [next, end) (uniform)
    if (tid == 0) mbar_init(bar);

    for (;;) {
        __syncthreads();
        if (tid == 0) sScal[0] = atomicAdd(&p.sc.words[0], 1);
        __syncthreads();
        const int u = sScal[0];
        if (u >= p.n_units) break;
        const int k = find_image(p.n_img, u, [&](int i) { return p.img[i].unit_base; });
        const DetImage& im = p.img[k];
        const void* src = im.src;
        const long long pitch = im.pitch;
        const int H = im.H, W = im.W, dtype = im.dtype;
        const int local = u - im.unit_base;
        const int sr = local / im.nsc, sc = local - sr * im.nsc;
        const int ys = sr * im.S, x0 = sc * kInner;
        const int S_act = min(im.S, H - ys);
        if (im.wait_slot > 0) {  // pixels still arriving: wait for the group (uniform across the CTA)
            if (tid == 0)
                sScal[2] = wait_ready(p.ready + (im.wait_slot - 1), p.ready_epoch, p.ready_spins, p.sc.words) ? 1 : 0;
            __syncthreads();
            if (!sScal[2]) {
                // the copy never arrived: the unit finds no edgels (its row
                // segments are written empty, so the ordering pass reads no
                // stale entries) and the call reports TOED_ERR_TIMEOUT
                for (int i = tid; i < 2 * S_act; i += kThreads)
                    if (TOED_IN_BOUNDS(im.seg_base + (long long)(2 * ys + i) * im.nsc + sc < p.sc.seg_cap, p.sc.words))
                        p.sc.seg[im.seg_base + (long long)(2 * ys + i) * im.nsc + sc] = make_int2(0, 0);
                continue;
            }
        }
        const int nsteps = (2 * S_act + 3 + 2 * B - 1) / (2 * B);
        const int W2 = 2 * W;
        const int row_lo = max(p.border, 2 * ys), row_hi = min(2 * H - p.border, 2 * ys + 2 * S_act);
        const int col_lo = p.border, col_hi = W2 - p.border;
        const long long seg0 = im.seg_base;
        const int xin = x0 - R - 2;  // image column of sIn column 0
        int x_al = xin, shift = 0;
        if (!ASYNC && im.tma == 1) {
            const int al = im.tma_align;
            x_al = (xin >= 0) ? (xin / al) * al : -(((-xin) + al - 1) / al) * al;  // floor to the alignment
            shift = xin - x_al;
        }
        const int rawpitch = im.tma_boxw * (dtype == TOED_U8 ? 1 : 4);  // bytes per staged row
        const int gc_base = 2 * (x0 - 1);

        // 2x-grid rows 0 and 1 of the NMS window start empty
        for (int i = tid; i < 2 * kFxyStride; i += kThreads) sFxy[i] = make_float2(0.f, 0.f);
        if (tid < 4 * kHalves) sMask[tid] = 0u;

        // async row staging: this thread's chunk of every box, fixed for the unit
        AsyncLane alane{};
        if (ASYNC && im.tma == 2) alane = async_lane<R>(static_cast<const float*>(src), pitch, W, xin);
        int rb = 0;
        for (int s = 0; s < nsteps; ++s) {
            // logical slot h <-> ring row (rb + h) mod RING <-> ext row
            // s*B - R - 2 + h <-> image row ys - 1 + ext row
            // ---- 1. input rows -> input ring (FP32, zero padded) -----------
            if (ASYNC && im.tma == 2) {
                stage_rows_async<R>(sIn, sRaw, static_cast<const float*>(src), pitch, H, alane, ys, s, nsteps, rb,
                                    p.sc.words);
                __syncthreads();  // every thread's rows are in before the row pass
            } else if (!ASYNC && im.tma == 1) {
                // rows arrive by TMA (out-of-image texels read as zero, the
                // reference's zero padding); step s+1's box is requested as
                // soon as step s has consumed the staging buffer
                const int nch = (s == 0) ? (C::HS + B - 1) / B : 1;
                for (int ch = 0; ch < nch; ++ch) {
                    const int row0 = (s == 0) ? ys - R - 3 + ch * B : ys + s * B + R;
                    // the first prologue box; later boxes are requested at the end of
                    // the previous chunk, steady-state boxes at the end of the previous step
                    if (s == 0 && ch == 0 && tid == 0)
                        tma_load_rows(&p.tmap[k], smem_addr(sRaw), bar, x_al, row0, (uint32_t)(B * rawpitch));
                    // no barrier before the conversion: the input ring rows it
                    // writes are read only by this step's row pass, so threads
                    // still busy with the previous step's gather join late
                    const bool ok = mbar_wait(bar, phase);
                    phase ^= 1u;
                    const int nrows = min(B, C::HS - ((s == 0) ? ch * B : 0));
                    const int a0 = (s == 0) ? ch * B : rb + 2 * R + 3;  // ring row of box row 0 (before wrapping)
                    if (ok) {
                        // a warp per staged row, lanes along it
                        if (dtype == TOED_U8) {
                            for (int rr = wid; rr < nrows; rr += kThreads / 32) {
                                float* dst = sIn + ring_wrap<C::RING>(a0 + rr) * C::NIN;
                                const unsigned char* srow = sRaw + rr * rawpitch + shift;
                                for (int cc = lane; cc < C::NIN; cc += 32)
                                    if (TOED_IN_BOUNDS(rr * rawpitch + shift + cc < (int)C::sz_raw, p.sc.words))
                                        dst[cc] = (float)srow[cc];
                            }
                        } else if ((R & 1) == 0) {
                            // even r: the staged row starts 8-byte aligned (shift = xin mod 4 is even)
                            const float* rf = reinterpret_cast<const float*>(sRaw);
                            static_assert(C::NIN % 2 == 0 && C::NIN / 2 <= 32, "one float2 per lane");
                            for (int rr = wid; rr < nrows; rr += kThreads / 32) {
                                float2* dst = reinterpret_cast<float2*>(sIn + ring_wrap<C::RING>(a0 + rr) * C::NIN);
                                const float2* srow = reinterpret_cast<const float2*>(rf + rr * im.tma_boxw + shift);
                                if (lane < C::NIN / 2 &&
                                    TOED_IN_BOUNDS((rr * im.tma_boxw + shift) * 4 + 8 * lane + 8 <= (int)C::sz_raw,
                                                   p.sc.words))
                                    dst[lane] = srow[lane];
                            }
                        } else {
                            const float* rf = reinterpret_cast<const float*>(sRaw);
                            for (int rr = wid; rr < nrows; rr += kThreads / 32) {
                                float* dst = sIn + ring_wrap<C::RING>(a0 + rr) * C::NIN;
                                const float* srow = rf + rr * im.tma_boxw + shift;
                                for (int cc = lane; cc < C::NIN; cc += 32)
                                    if (TOED_IN_BOUNDS((rr * im.tma_boxw + shift + cc) * 4 + 4 <= (int)C::sz_raw,
                                                       p.sc.words))
                                        dst[cc] = srow[cc];
                            }
                        }
                    }
                    if (__syncthreads_or(!ok)) {
                        // give up on this CTA: flag it, drain the copy in flight, leave
                        if (tid == 0) atomicOr(&p.sc.words[2], TOED_FLAG_TIMEOUT);
                        mbar_wait(bar, phase ^ 1u);
                        return;
                    }
                    if (s == 0 && ch + 1 < nch && tid == 0)
                        tma_load_rows(&p.tmap[k], smem_addr(sRaw), bar, x_al, row0 + B, (uint32_t)(B * rawpitch));
                }
                // the next step's rows (the last prologue chunk has been consumed)
                if (s + 1 < nsteps && tid == 0)
                    tma_load_rows(&p.tmap[k], smem_addr(sRaw), bar, x_al, ys + (s + 1) * B + R,
                                  (uint32_t)(B * rawpitch));
            } else {
                const int nrows = (s == 0) ? C::HS : B;
                const int a0 = (s == 0) ? 0 : rb + 2 * R + 3;
                const int img_row0 = (s == 0) ? ys - R - 3 : ys + s * B + R;
                for (int i = tid; i < nrows * C::NIN; i += kThreads) {
                    const int rr = i / C::NIN, cc = i - rr * C::NIN;
                    if (TOED_IN_BOUNDS(ring_wrap<C::RING>(a0 + rr) < C::RING, p.sc.words))
                        sIn[ring_wrap<C::RING>(a0 + rr) * C::NIN + cc] =
                            fetch_px(src, pitch, H, W, dtype, img_row0 + rr, xin + cc);
                }
                __syncthreads();
            }
            // ---- 2. row pass ------------------------------------------------
            if (s == 0) {
                row_pass<R>(sIn, 0, C::HS, sP, tp, p.sc.words);
            } else {
                row_pass<R>(sIn, ring_wrap<C::RING>(rb + 2 * R + 3), B, sP, tp, p.sc.words);
                // the previous step's last two 2x rows become rows 0 and 1
                for (int i = tid; i < 2 * kFxyStride; i += kThreads) sFxy[i] = sFxy[2 * B * kFxyStride + i];
                if (tid < 4 * kHalves) sMask[tid] = sMask[2 * B * 2 * kHalves + tid];
            }
            __syncthreads();
            // ---- 3. column pass: Ix, Iy for 2x rows m = 2..2B+1, and the
            // threshold test as ballots over the strip's columns
            const int gr_base = 2 * ys - 4 + 2 * s * B;  // global 2x row of NMS row m: gr_base + m
            {
                // warp -> (sub-grid, 8-row group, 32-column half of the strip)
                const int sg = wid & 3, g = (wid >> 2) & 1, h = wid >> 3;
                const int a = sg >> 1, b = sg & 1;
                const int col = 32 * h + lane;  // ext column
                float fx[kColRows], fy[kColRows];
                // sub-grid (a, b): x taps T / F / S for (0,0) / (1,0) / (.,1),
                // y taps truncated for (0,0), full for (0,1), shifted for (1,.)
                const float2* P = sP + (sg == 0 ? 0 : (sg == 2 ? 1 : 2)) * C::RING * C::PS;
                if (sg == 0)
                    col_pass<R, 0>(P, rb, g, col, tp, fx, fy);
                else if (sg == 1)
                    col_pass<R, 1>(P, rb, g, col, tp, fx, fy);
                else
                    col_pass<R, 2>(P, rb, g, col, tp, fx, fy);
                const int c = 2 * col + b, Gc = gc_base + c;
                // the strip's output columns inside the image's border (lanes)
                const unsigned colmask =
                    __ballot_sync(0xffffffffu, col >= 1 && col <= kInner && Gc >= col_lo && Gc < col_hi);
#pragma unroll
                for (int o = 0; o < kColRows; ++o) {
                    const int m = 2 * (g * kColRows + o) + a + 2;
                    const float2 f = make_float2(fx[o], fy[o]);
                    if (TOED_IN_BOUNDS(m < C::MS && c < C::FW, p.sc.words)) sFxy[m * kFxyStride + c] = f;
                    const int Gr = gr_base + m;  // the same for the whole warp
                    // cpu_toed.cpp:403 as a prefilter on the squared magnitude (thr2 a
                    // little below thr^2, so the list holds every point nms_eval's exact
                    // test `|grad I| > thr` keeps; no square root per point)
                    const unsigned bal = __ballot_sync(0xffffffffu, fmaf(f.x, f.x, f.y * f.y) > p.thr2) &
                                         ((Gr >= row_lo && Gr < row_hi) ? colmask : 0u);
                    if (lane == 0) sMask[(m * 2 + b) * kHalves + h] = bal;
                }
            }
            if (tid < 32) sAccCnt[tid] = 0;
            __syncthreads();
            // ---- 4a. points above the threshold, listed in row-major order ---
            // NMS rows m = 1..2B; mask (m, parity, half): bit L <-> 2x column
            // 2 (32 half + L) + parity.  Every warp counts and scans the rows
            // itself (lane L <-> row L + 1): no barrier between the scan and
            // the list writes.
            int row_excl, LA;
            {
                int cnt = 0;
#pragma unroll
                for (int q = 0; q < 2 * kHalves; ++q) cnt += __popc(sMask[(lane + 1) * 2 * kHalves + q]);
                int incl = cnt;
#pragma unroll
                for (int d = 1; d < 32; d <<= 1) {
                    const int y = __shfl_up_sync(0xffffffffu, incl, d);
                    if (lane >= d) incl += y;
                }
                row_excl = incl - cnt;
                LA = __shfl_sync(0xffffffffu, incl, 31);
            }
            {
                const unsigned lt = (1u << lane) - 1u;
                for (int m = 1 + wid; m <= 2 * B; m += kThreads / 32) {
                    int pos0 = __shfl_sync(0xffffffffu, row_excl, m - 1);
#pragma unroll
                    for (int h = 0; h < kHalves; ++h) {
                        const unsigned mk0 = sMask[(m * 2) * kHalves + h], mk1 = sMask[(m * 2 + 1) * kHalves + h];
                        const bool k0 = (mk0 >> lane) & 1u, k1 = (mk1 >> lane) & 1u;
                        const int pos = pos0 + __popc(mk0 & lt) + __popc(mk1 & lt);
                        const unsigned c0 = 2 * (32 * h + lane);
                        if (k0 && TOED_IN_BOUNDS(pos < C::MAXC, p.sc.words)) sList[pos] = ((unsigned)m << 8) | c0;
                        if (k1 && TOED_IN_BOUNDS(pos + (k0 ? 1 : 0) < C::MAXC, p.sc.words))
                            sList[pos + (k0 ? 1 : 0)] = ((unsigned)m << 8) | (c0 + 1);
                        pos0 += __popc(mk0) + __popc(mk1);
                    }
                }
            }
            __syncthreads();
            // ---- 4b. NMS on the list with full warps; survivors compacted in
            // place, order kept (their rank never exceeds their list position).
            // One barrier per round: the warp counts alternate between two
            // halves of sWarp.
            int nacc = 0;
            for (int r0 = 0, rd = 0; r0 < LA; r0 += kThreads, rd ^= 1) {
                const int e = r0 + tid;
                unsigned rec = 0;
                bool acc = false;
                if (e < LA) {
                    rec = sList[e];
                    if (NMSTO) {
                        const int m = rec >> 8, c = rec & 255;
                        float d7[7], tx, ty;
                        gather_hi<R>(sP, sTab, rb, m, c, d7, p.sc.words);
                        const float2 g = sFxy[m * kFxyStride + c];
                        to_vec32(g.x, g.y, d7, &tx, &ty);
                        acc = nms_eval<true>(sFxy, m, c, p.thr, tx, ty, p.sc.words).cand;
                    } else {
                        acc = nms_decide(sFxy, rec >> 8, rec & 255, p.thr, p.sc.words);
                    }
                }
                const unsigned bal = __ballot_sync(0xffffffffu, acc);
                int* wc = sWarp + (kThreads / 32) * rd;
                if (lane == 0) wc[wid] = __popc(bal);
                __syncthreads();
                // every warp scans the warp counts (lane w <-> warp w)
                constexpr int NWARP = kThreads / 32;
                const int wx = (lane < NWARP) ? wc[lane] : 0;
                int wincl = wx;
#pragma unroll
                for (int d = 1; d < NWARP; d <<= 1) {
                    const int y = __shfl_up_sync(0xffffffffu, wincl, d);
                    if (lane >= d) wincl += y;
                }
                const int off = __shfl_sync(0xffffffffu, wincl - wx, wid);
                const int tot = __shfl_sync(0xffffffffu, wincl, NWARP - 1);
                if (acc) {
                    const int dpos = nacc + off + __popc(bal & ((1u << lane) - 1u));
                    if (TOED_IN_BOUNDS(dpos < C::MAXC, p.sc.words)) sList[dpos] = rec;
                    atomicAdd(&sAccCnt[(rec >> 8) - 1], 1);
                }
                nacc += tot;
            }
            __syncthreads();
            // ---- 4c. staging slots: carved from this CTA's reserved range
            // (tracked identically by every thread), refilled from the global
            // cursor only when a step does not fit
            if (nacc > 0 && stg_next + nacc > stg_end) {
                const int n = max(p.stage_blk, nacc);
                if (tid == 0) sScal[1] = atomicAdd(&p.sc.words[1], n);
                __syncthreads();
                stg_next = sScal[1];
                stg_end = stg_next + n;
            }
            const int base = stg_next;
            stg_next += nacc;
            if (tid == 0 && (long long)base + nacc > p.sc.staging_cap) atomicOr(&p.sc.words[2], TOED_FLAG_STAGING_FULL);
            // warp 0: the row-segment table {staging offset, count} per 2x row,
            // while the other warps gather the edgels
            if (wid == 0) {
                const int cnt = sAccCnt[lane];
                int incl = cnt;
#pragma unroll
                for (int d = 1; d < 32; d <<= 1) {
                    const int y = __shfl_up_sync(0xffffffffu, incl, d);
                    if (lane >= d) incl += y;
                }
                const int Gr = gr_base + lane + 1;
                if (Gr >= 2 * ys && Gr < 2 * ys + 2 * S_act)
                    if (TOED_IN_BOUNDS(seg0 + (long long)Gr * im.nsc + sc < p.sc.seg_cap, p.sc.words))
                        p.sc.seg[seg0 + (long long)Gr * im.nsc + sc] = make_int2(base + incl - cnt, cnt);
            }
            // ---- 5. per edgel: the seven higher derivatives from the row-pass
            // ring into a deferred record (the epilogue runs when the
            // ring of records is full)
            {
                for (int j0 = 0; j0 < nacc;) {
                    const int chunk = min(nacc - j0, C::NREC - nrec);
                    for (int j = tid - 32; wid > 0 && j < chunk; j += kThreads - 32) {
                        const unsigned rec = sList[j0 + j];
                        const int m = rec >> 8, c = rec & 255;
                        float d7[7];
                        gather_hi<R>(sP, sTab, rb, m, c, d7, p.sc.words);
                        const float fxx = d7[0], fxy = d7[1], fyy = d7[2], fxxy = d7[3], fxyy = d7[4],
                                    fxxx = d7[5], fyyy = d7[6];
                        NmsEval e;
                        if (NMSTO) {
                            const float2 g = sFxy[m * kFxyStride + c];
                            float tx, ty;
                            to_vec32(g.x, g.y, d7, &tx, &ty);
                            e = nms_eval<true>(sFxy, m, c, p.thr, tx, ty);
                        } else {
                            e = nms_eval(sFxy, m, c, p.thr);
                        }
                        const int Gr = gr_base + m, Gc = gc_base + c;
                        if (!TOED_IN_BOUNDS(nrec + j < C::NREC, p.sc.words)) continue;
                        float* rc = sRec + (nrec + j) * C::RECW;
                        rc[0] = e.gx; rc[1] = e.gy; rc[2] = e.mv; rc[3] = e.nx; rc[4] = e.ny; rc[5] = e.slope;
                        rc[6] = e.Map; rc[7] = e.Mdp; rc[8] = e.Mam; rc[9] = e.Mdm;
                        rc[10] = fxx; rc[11] = fxy; rc[12] = fyy; rc[13] = fxxy; rc[14] = fxyy; rc[15] = fxxx;
                        rc[16] = fyyy;
                        rc[17] = __int_as_float(Gr);
                        rc[18] = __int_as_float(Gc);
                        rc[19] = __int_as_float(base + j0 + j);
                        rc[20] = __int_as_float(k);
                    }
                    nrec += chunk;
                    j0 += chunk;
                    if (nrec == C::NREC) {
                        __syncthreads();
                        for (int r = tid; r < nrec; r += kThreads) {
                            const float* rc = sRec + r * C::RECW;
                            finish_edgel<HYB>(rc, p.sc, 2 * p.img[__float_as_int(rc[20])].W);
                        }
                        nrec = 0;
                        __syncthreads();
                    }
                }
            }
            // (no barrier here: the next step's first barrier, before its row
            // pass and its carry of rows 0 and 1, orders this step's reads)
            rb = ring_wrap<C::RING>(rb + B);
        }
    }
    // flush the records still in the ring (the loop exit follows a barrier)
    for (int r = tid; r < nrec; r += kThreads) {
        const float* rc = sRec + r * C::RECW;
        finish_edgel<HYB>(rc, p.sc, 2 * p.img[__float_as_int(rc[20])].W);
    }
}


}  // namespace toed
