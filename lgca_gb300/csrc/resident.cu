// Resident form of the lattice step: for lattices whose one-step warp tasks
// (two words per lane, one row per warp) all fit on the GPU at once, e.g.
// FHP-III 8192 x 2048 = 4096 warps on 152 SMs.  One cooperative launch
// advances nsteps steps; the state never goes back to global memory between
// them.
//
// Reference: OMP_Lattice<M>::collide_and_propagate, keva92/lgca
// src/omp_lattice.cpp:100-249 (the pull table and rules are those of
// step_body.cuh, which states them per model and row parity).
//
// Decomposition.  Block b owns the band of rows [H*b/nb, H*(b+1)/nb); warp
// (r, h) of the block owns pairs 32h .. 32h+31 of band row r.  Between steps
// a warp keeps the channels its own row pulls from itself (FHP 0, 3 and the
// rest channel 6; HPP 0 and 2) in registers, and writes every moving channel
// of its pair to the block's shared memory, from which the rows above and
// below, and the lanes at its ends, pull:
//   FHP: row y-1 gives channels 1, 2; row y+1 gives 4, 5
//   HPP: row y-1 gives channel 1;     row y+1 gives 3
// A band's first and last rows also pull from the neighbouring bands: each
// block writes its first row's "from below" channels and its last row's
// "from above" channels to a halo slot in global memory (three slots per
// block and side, by step modulo 3), and the edge warps of the neighbouring
// block load them from there.  Every word goes out as two 64-bit items, one
// half of the word in the low 32 bits and the step it belongs to in the high
// 32 bits; an item is written and read whole (single-copy atomic), so a
// reader that sees the step it wants has the data, with no fence and no
// separate flag between writer and reader.  Interior rows never wait for
// another block.  A writer overwrites a slot three steps later, by which
// time every reader of the old contents has moved on: the writer has read
// the step in between from one of the readers' warps, which had waited for
// all warps of its row to publish that step (through the block barrier, or
// its row's barrier below).
//
// Forcing belongs to the start of a step (it flips source words before the
// pull).  Here the owner of the forcing column applies the flips of step j+1
// to its registers at the end of step j, before it writes them to shared
// memory, so that every lane that pulls the forced words sees them; the
// state written back to global memory after the last step carries no flips.
//
// Input and output may also be in the reference's byte-per-cell layout
// (lgca_run_job_async): each lane converts its own 128 cells in the launch's
// first and last moments, so no conversion kernel runs between jobs.
//
// The launcher takes the fewest bands of the smallest height the SMs allow,
// which leaves a few SMs free for other streams' kernels.
//
// Synchronisation per step, one of two kinds (template parameter RS):
//  - a block barrier;
//  - row barriers (RS): each band row has two mbarriers in shared memory, by
//    step parity, on which all lanes of the row's warps arrive once they
//    have written a step's channels; before a step a warp waits for that
//    step on its own row's and its band neighbour rows' barriers.  A warp is
//    then at most one step ahead of the rows it pulls from, and a buffer is
//    rewritten only after its readers have published the step that followed
//    their reads.  Warps drift apart within those bounds, so warps with more
//    work (walls, the obstacle, the forcing column, band edges) do not hold
//    up the whole block every step.  Measured on GB300 it pays for
//    FHP-II/III on blocks of 24 warps or more, which the launcher gives it.
// The band's edge warps also wait for their halo items.  Every wait is
// bounded (wait_ns, measured with %globaltimer): past it, or when another
// warp or block has given up, a warp records the error in *err, finishes the
// step without further waits, and the block returns after its next barrier.
// *err is sticky: a launch that finds it set does nothing.
#include "step_body.cuh"

#include <algorithm>

namespace lgca_gpu {

static constexpr int RES_MAX_WARPS = 28;  // warps per block (<= 72 registers per thread)

struct ResidentArgs {
    // [3 steps][nblk][2 sides][2 channels][nw][2] items; items of time t
    // carry the tag (epoch << 24) | (t + 1), and no item in the slots may
    // carry a tag of this launch's epoch when it starts
    uint64_t *halo;
    unsigned epoch;  // 1 .. 255
    int *err;
    uint64_t seed, t0;
    int nsteps;
    int nblk, wpr, rpb;  // blocks, warps per row, most rows in a band
    uint64_t wait_ns;
    int withhold;  // block that never writes its halo slots (test hook), -1 none
    // optional byte-per-cell state (the reference's layout: H rows of W
    // bytes, bit d = channel d): the launch reads its input from aos_in
    // instead of a.src, and writes its result to aos_out as well as to a.dst
    const uint8_t *aos_in;
    uint8_t *aos_out;
    // optional B x B block sums of the result (B = sums_B in 8, 16, 32, 64;
    // 0: none) added into N, Jx2, Jy (Wb = ceil(W / B) columns), which must
    // be zero before the launch
    int sums_B, sums_Wb;
    int32_t *sums_N, *sums_Jx2, *sums_Jy;
};

// Byte-per-cell <-> bit-plane conversion of 8 cells (the 8 bytes of x, cell
// i in byte i).  gather8: bit i of the result = bit d of byte i (the
// masked bits sit 8 apart, and one multiply moves bit 8i to bit 56 + i;
// every partial product lands on its own bit, so nothing carries into the
// top byte).  spread8: byte i of the result = bit i of b (b copied into
// every byte, byte i masked to bit i, then a byte-wise "is non-zero" by
// adding 0x7f, which cannot carry out of a byte).
LGCA_HDI uint64_t res_gather8(uint64_t x, int d)
{
    return (((x >> d) & 0x0101010101010101ull) * 0x0102040810204080ull) >> 56;
}
LGCA_HDI uint64_t res_spread8(uint64_t b)
{
    const uint64_t x = (b * 0x0101010101010101ull) & 0x8040201008040201ull;
    return ((x + 0x7f7f7f7f7f7f7f7full) >> 7) & 0x0101010101010101ull;
}

static constexpr int RES_HALO_SLOTS = 3;
static constexpr int RES_KEYS = 16;  // steps of random keys a warp draws at once
static constexpr int RES_ROWSYNC_WARPS = 24;  // FHP-II/III blocks from this many warps use row barriers

// Shared memory of a block, in words: 8 control words, two row-barrier
// words per band row, a key ring of 2 x RES_KEYS words per warp, then the
// two step buffers of rpb x SP x nw words.
LGCA_HDI size_t res_smem_words(int SP, int nw, int rpb, int wpr)
{
    return 8 + 2 * (size_t)rpb + 2 * RES_KEYS * (size_t)rpb * wpr + 2 * (size_t)rpb * SP * nw;
}

// Particle count and momentum of the cells in mask m of the words v (the
// block-sum weights: FHP Jx2 = 2n0 + n1 - n2 - 2n3 - n4 + n5 in units of
// 1/2, Jy = n1 + n2 - n4 - n5 in units of sin 60; HPP Jx2 = 2(n0 - n2),
// Jy = n1 - n3; src/lgca_models.h:51-52, :246).
template <int MODEL>
__device__ __forceinline__ void res_counts(const uint64_t *v, uint64_t m, int &n, int &jx2, int &jy)
{
    constexpr int D = ModelTraits<MODEL>::D;
    int c[7];
#pragma unroll
    for (int d = 0; d < D; ++d) c[d] = __popcll(v[d] & m);
    n = 0;
#pragma unroll
    for (int d = 0; d < D; ++d) n += c[d];
    if (MODEL == M_HPP) {
        jx2 = 2 * (c[0] - c[2]);
        jy = c[1] - c[3];
    } else {
        jx2 = 2 * c[0] + c[1] - c[2] - 2 * c[3] - c[4] + c[5];
        jy = c[1] + c[2] - c[4] - c[5];
    }
}

#ifndef LGCA_HOST_EMULATION
// the block's shared memory: 8 control words, then two buffers of
// rpb x SP x nw words
__device__ __forceinline__ uint64_t *res_smem()
{
    extern __shared__ uint4 res_sm[];
    return reinterpret_cast<uint64_t *>(res_sm);
}
// two halo items (each 64-bit access single-copy atomic, coherent at GPU scope)
__device__ __forceinline__ ulonglong2 ld_items(const uint64_t *p)
{
    ulonglong2 v;
    asm volatile("ld.relaxed.gpu.global.v2.u64 {%0, %1}, [%2];" : "=l"(v.x), "=l"(v.y) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_items(uint64_t *p, uint64_t a, uint64_t b)
{
    asm volatile("st.relaxed.gpu.global.v2.u64 [%0], {%1, %2};" ::"l"(p), "l"(a), "l"(b) : "memory");
}
// mbarrier in shared memory: init with the arrivals of a phase, arrive
// (release), and test whether the phase of the given parity has completed
// (acquire)
__device__ __forceinline__ void res_bar_init(uint64_t *bar, unsigned count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"((unsigned)__cvta_generic_to_shared(bar)),
                 "r"(count)
                 : "memory");
}
__device__ __forceinline__ void res_bar_arrive(uint64_t *bar)
{
    asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.shared::cta.b64 st, [%0];\n\t}" ::"r"(
                     (unsigned)__cvta_generic_to_shared(bar))
                 : "memory");
}
__device__ __forceinline__ bool res_bar_done(const uint64_t *bar, unsigned parity)
{
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"((unsigned)__cvta_generic_to_shared(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
__device__ __forceinline__ uint64_t res_timer_ns()
{
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
#endif

template <int MODEL>
struct ResPlanes {
    static constexpr bool HPP = MODEL == M_HPP;
    static constexpr int SP = HPP ? 4 : 6;     // moving channels (kept in shared memory)
    static constexpr int NV = HPP ? 1 : 2;     // channels pulled from each of rows y-1, y+1
    static constexpr int A0 = 1;               // first channel from row y-1 (then A0 + 1 for FHP)
    static constexpr int B0 = HPP ? 3 : 4;     // first channel from row y+1
    static constexpr int WEST = HPP ? 2 : 3;   // the forcing's west-moving channel
};

template <int MODEL, int GM, bool RS>
__global__ void __launch_bounds__(32 * RES_MAX_WARPS, 1)
    k_resident(const __grid_constant__ StepArgs a, const __grid_constant__ ResidentArgs R)
{
    using P = ResPlanes<MODEL>;
    constexpr int D = ModelTraits<MODEL>::D;
    constexpr int SP = P::SP, NV = P::NV, A0 = P::A0, B0 = P::B0, WEST = P::WEST;
    uint64_t *const sm = res_smem();
    // control words: the stop flags [4..5].  With a block barrier per step
    // they go by step parity: a stop flag is written before the barrier that
    // ends its step and read by every warp right after it; the slot is not
    // written again until every warp has passed the next barrier, so all
    // warps of the block read the same value and return together.  With row
    // barriers, [4] is read once after the step loop.  The check before the
    // first step uses slot 1.
    volatile uint64_t *const ctl = sm;
    uint64_t *const bars = sm + 8;  // row barriers [band row][step parity] (RS)
    // each warp's random keys: the chirality keys of RES_KEYS steps, then the
    // forcing keys of the steps after them, drawn by its lanes at once
    // (lane i < RES_KEYS: chirality of step j + i; lane RES_KEYS + i:
    // forcing of step j + i + 1), so that no warp draws keys alone on the
    // path to the step barrier
    uint64_t *const keyring = bars + 2 * R.rpb;
    uint64_t *const rows = keyring + (size_t)2 * RES_KEYS * R.rpb * R.wpr;
    const PlaneGeom &g = a.g;
    const int nw = g.nw, np = nw >> 1;
    const size_t ps = g.ps;
    const size_t bufw = (size_t)R.rpb * SP * nw, roww = (size_t)SP * nw;
    const int nb = R.nblk, b = blockIdx.x;
    const int bl = b == 0 ? nb - 1 : b - 1, br = b == nb - 1 ? 0 : b + 1;
    const int y0 = (int)((long long)g.H * b / nb), y1 = (int)((long long)g.H * (b + 1) / nb);
    const int nrows = y1 - y0;
    const int lane = threadIdx.x, warp = threadIdx.y;
    const int r = warp / R.wpr, hw = warp - r * R.wpr;
    const int t = hw * 32 + lane, w0 = 2 * t;
    const bool rowok = r < nrows;  // warp-uniform
    const bool active = rowok && t < np;
    const int y = y0 + (rowok ? r : 0);
    const bool even = (y & 1) == 0;
    const bool top = rowok && r == 0, bot = rowok && r == nrows - 1;
    const bool need_w = active && lane == 0;
    const bool need_e = active && (lane == 31 || t == np - 1);
    const int widx = t == 0 ? nw - 1 : w0 - 1;
    const int eidx = t == np - 1 ? 0 : w0 + 2;
    const unsigned row0 = (unsigned)y * (unsigned)g.pitch;
    const int fw = a.fx >> 6;
    const bool fowner = a.force_thr != 0 && active && (fw >> 1) == t;
    // slot of the halo items of time `tm` of side `side` (0: first row, 1: last row) of block blk
    auto halo_slot = [&](unsigned tm, int blk, int side) -> uint64_t * {
        return R.halo + (size_t)(((int)(tm % RES_HALO_SLOTS) * nb + blk) * 2 + side) * 2 * nw * 2;
    };

    if (warp == 0 && lane == 0) {
        ctl[4] = 0;
        ctl[5] = (uint64_t)(*(volatile int *)R.err);
        if (RS)
            for (int i = 0; i < 2 * R.rpb; ++i) res_bar_init(bars + i, 32u * (unsigned)R.wpr);
    }
    if (RS) __syncthreads();  // the barriers are set up before anyone arrives

    // the row's state at the launch's first step
    uint64_t s[2][7] = {};
    uint64_t solid[2] = {0, 0}, slip[2] = {0, 0};
    // input in the byte-per-cell layout: each lane converts its pair's 128
    // cells (8 x 16 bytes) into planes written to a.dst, which this launch
    // otherwise touches only with its result, and then loads them back as
    // planes like any other input (the conversion's registers stay out of
    // the steps' register allocation)
    const uint64_t *in = a.src;
    if (R.aos_in) {
        if (active) {
            const uint4 *cells =
                reinterpret_cast<const uint4 *>(R.aos_in + (size_t)y * (size_t)g.W + (size_t)128 * t);
#pragma unroll
            for (int k = 0; k < 2; ++k) {
                uint64_t wd[7] = {};
#pragma unroll
                for (int q = 0; q < 4; ++q) {  // cells 64k + 16q .. 64k + 16q + 15
                    const uint4 v = __ldcg(cells + 4 * k + q);
                    const uint64_t lo = ((uint64_t)v.y << 32) | v.x, hi = ((uint64_t)v.w << 32) | v.z;
#pragma unroll
                    for (int d = 0; d < D; ++d)
                        wd[d] |= (res_gather8(lo, d) | (res_gather8(hi, d) << 8)) << (16 * q);
                }
#pragma unroll
                for (int d = 0; d < D; ++d) a.dst[d * ps + row0 + w0 + k] = wd[d];
            }
        }
        asm volatile("" ::: "memory");
        in = a.dst;
    }
    if (active) {
#pragma unroll
        for (int d = 0; d < D; ++d) {
            const ulonglong2 v = __ldcg(reinterpret_cast<const ulonglong2 *>(in + d * ps + row0 + w0));
            s[0][d] = v.x;
            s[1][d] = v.y;
        }
    }
    if (active) {
        if (GM >= GEOM_NOSLIP) {
            const ulonglong2 v = __ldg(reinterpret_cast<const ulonglong2 *>(a.solid + row0 + w0));
            solid[0] = v.x;
            solid[1] = v.y;
        }
        if (GM == GEOM_FULL) {
            const ulonglong2 v = __ldg(reinterpret_cast<const ulonglong2 *>(a.slip + row0 + w0));
            slip[0] = v.x;
            slip[1] = v.y;
        }
    }
    // warps without wall or obstacle cells skip the boundary multiplexer
    const bool walls = GM != GEOM_NONE &&
                       __any_sync(FULL, (solid[0] | solid[1] | slip[0] | slip[1]) != 0ull);

    // the forcing draw of a step: does the forcing column flip in this row
    // (the owner of the column's word only)
    auto force_draw = [&](uint64_t fkey) -> bool {
        if (!fowner) return false;
        const uint64_t u = lgca_rng_draw(fkey, lgca_rng_index((uint32_t)y, (uint32_t)a.fx)) >> 32;
        return u < a.force_thr;
    };
    // that flip applied to the registers: a fluid cell with channel 0 empty
    // and the west-moving channel occupied reverses it
    auto force = [&](bool flip) {
        if (!flip) return;
        const uint64_t bit = 1ull << (a.fx & 63);
        const uint64_t m0 = (fw & 1) ? 0ull : bit, m1 = (fw & 1) ? bit : 0ull;
        const uint64_t f0 = ~s[0][0] & s[0][WEST] & ~solid[0] & ~slip[0] & m0;
        const uint64_t f1 = ~s[1][0] & s[1][WEST] & ~solid[1] & ~slip[1] & m1;
        s[0][0] |= f0;
        s[0][WEST] &= ~f0;
        s[1][0] |= f1;
        s[1][WEST] &= ~f1;
    };
    // the moving channels of time `tm` to shared memory buffer tm & 1; the
    // band's edge rows also to their halo slots
    auto publish = [&](unsigned tm) {
        if (!active) return;
        uint64_t *dr = rows + (tm & 1) * bufw + (size_t)r * roww;
#pragma unroll
        for (int d = 0; d < SP; ++d)
            *reinterpret_cast<ulonglong2 *>(dr + (size_t)d * nw + w0) = make_ulonglong2(s[0][d], s[1][d]);
        if (b == R.withhold) return;
        const uint64_t tag = (uint64_t)((R.epoch << 24) | (tm + 1)) << 32;
        auto put = [&](uint64_t *slot, int k, uint64_t v0, uint64_t v1) {
            uint64_t *p = slot + ((size_t)k * nw + w0) * 2;
            st_items(p, tag | (v0 & 0xffffffffull), tag | (v0 >> 32));
            st_items(p + 2, tag | (v1 & 0xffffffffull), tag | (v1 >> 32));
        };
        if (top) {  // row y0: channels the last row of block bl pulls from below
            uint64_t *hs = halo_slot(tm, b, 0);
#pragma unroll
            for (int k = 0; k < NV; ++k) put(hs, k, s[0][B0 + k], s[1][B0 + k]);
        }
        if (bot) {  // row y1-1: channels the first row of block br pulls from above
            uint64_t *hs = halo_slot(tm, b, 1);
#pragma unroll
            for (int k = 0; k < NV; ++k) put(hs, k, s[0][A0 + k], s[1][A0 + k]);
        }
    };
    // publish; with row barriers every lane of the row's warps then arrives
    // on the row's barrier of that step's parity
    auto publish_arrive = [&](unsigned tm) {
        publish(tm);
        if (RS && rowok) res_bar_arrive(bars + 2 * r + (tm & 1));
    };
    // (row barriers) wait until this row and the band rows above and below
    // have published step j; false when the wait gave up (every lane returns
    // alike)
    auto rows_ready = [&](int j) -> bool {
        const unsigned par = (unsigned)(j >> 1) & 1u;
        const uint64_t *bj = bars + (j & 1);
        uint64_t t_start = 0;
        for (int spin = 0;; ++spin) {
            bool ok = res_bar_done(bj + 2 * r, par);
            if (!top) ok = ok && res_bar_done(bj + 2 * (r - 1), par);
            if (!bot) ok = ok && res_bar_done(bj + 2 * (r + 1), par);
            if (__all_sync(FULL, ok)) return true;
            if (spin == 0) t_start = res_timer_ns();
            const bool give_up =
                spin > 0 && (*(volatile int *)R.err || res_timer_ns() - t_start > R.wait_ns);
            if (__any_sync(FULL, give_up)) {
                if (lane == 0) atomicExch(R.err, 1);
                return false;
            }
        }
    };
    // an edge warp's words of time `tm` from a neighbour's halo slot: the
    // pair of each of its NV channels and, when `ek` >= 0, word `ew` of
    // channel slot ek (lanes with need_edge).  Polls until every item carries
    // the step; false when the wait gave up (every lane returns alike)
    auto halo_get = [&](const uint64_t *slot, unsigned tm, int ek, int ew, bool need_edge,
                        uint64_t (&v)[2][2], uint64_t &edge) -> bool {
        const uint64_t tag = (uint64_t)((R.epoch << 24) | (tm + 1));
        uint64_t t_start = 0;
        for (int spin = 0;; ++spin) {
            bool ok = true;
            if (active) {
#pragma unroll
                for (int k = 0; k < NV; ++k) {
                    const uint64_t *p = slot + ((size_t)k * nw + w0) * 2;
                    const ulonglong2 x = ld_items(p), y2 = ld_items(p + 2);
                    ok = ok && (x.x >> 32) == tag && (x.y >> 32) == tag && (y2.x >> 32) == tag &&
                         (y2.y >> 32) == tag;
                    v[0][k] = (x.x & 0xffffffffull) | (x.y << 32);
                    v[1][k] = (y2.x & 0xffffffffull) | (y2.y << 32);
                }
                if (ek >= 0 && need_edge) {
                    const ulonglong2 x = ld_items(slot + ((size_t)ek * nw + ew) * 2);
                    ok = ok && (x.x >> 32) == tag && (x.y >> 32) == tag;
                    edge = (x.x & 0xffffffffull) | (x.y << 32);
                }
            }
            if (__all_sync(FULL, ok)) return true;
            if (spin == 0) t_start = res_timer_ns();
            // the lanes decide together whether to give up
            const bool give_up =
                spin > 0 && (*(volatile int *)R.err || res_timer_ns() - t_start > R.wait_ns);
            if (__any_sync(FULL, give_up)) {
                if (lane == 0) atomicExch(R.err, 1);
                return false;
            }
            __nanosleep(32);
        }
    };

    force(force_draw(lgca_rng_key(R.seed, LGCA_STREAM_FORCE, R.t0)));
    publish_arrive(0u);
    __syncthreads();
    if (ctl[5]) return;  // an earlier launch gave up: do not step a partial state (block-uniform)

    const bool nsrow = (y == 0) || (y == g.H - 1);
    bool gave_up = false;  // this warp gave up a wait: it finishes the step without further waits
    uint64_t *const kr = keyring + (size_t)2 * RES_KEYS * warp;
    for (int j = 0; j < R.nsteps; ++j) {
        const int cur = j & 1;
        // (warp-uniform) with row barriers, warps past the band's last row
        // have nothing to wait for, and a warp that gave up stops here
        if (RS && (gave_up || !rowok)) break;
        if (j % RES_KEYS == 0) {
            __syncwarp();  // the ring's last keys have been read
            const int i = lane % RES_KEYS;
            kr[lane] = lane < RES_KEYS ? lgca_rng_key(R.seed, LGCA_STREAM_CHIR, R.t0 + (uint64_t)(j + i))
                                       : lgca_rng_key(R.seed, LGCA_STREAM_FORCE, R.t0 + (uint64_t)(j + i) + 1);
            __syncwarp();
        }
        // chirality key of step j, forcing key of step j + 1
        const uint64_t ck = kr[j % RES_KEYS], fk = kr[RES_KEYS + j % RES_KEYS];
        if (RS && !rows_ready(j)) gave_up = true;
        if (rowok) {  // (warp-uniform: warps past the band's last row only meet the block barrier)
            // the forcing draw of the next step, made now, off the step's end
            const bool flip_next = force_draw(fk);
            // chirality of word k of the pair, drawn (or, frozen, read) where it is used
            auto chirality = [&](int k) -> uint64_t {
                if (MODEL == M_HPP) return 0ull;
                if (a.chir) return __ldg(a.chir + row0 + w0 + k);
                return lgca_mix64(ck + lgca_rng_index((uint32_t)y, (uint32_t)(w0 + k)) * LGCA_RNG_GAMMA);
            };

            // ---- gather: own channels from registers, the others from rows y-1, y+1
            uint64_t n[2][7];
#pragma unroll
            for (int d = 0; d < D; ++d) {
                n[0][d] = s[0][d];
                n[1][d] = s[1][d];
            }
            // edge words in the order the pulls use them (step_body.cuh):
            //   FHP, even row: west 0 (row y), 1 (y-1), 5 (y+1); east 3 (row y)
            //   FHP, odd row:  west 0 (row y); east 3 (row y), 2 (y-1), 4 (y+1)
            //   HPP:           west 0 (row y); east 2 (row y)
            uint64_t eg[4] = {0, 0, 0, 0};
            const uint64_t *own = rows + cur * bufw + (size_t)r * roww;
            if (MODEL == M_HPP) {
                if (need_w) eg[0] = own[widx];
                if (need_e) eg[1] = own[(size_t)2 * nw + eidx];
            } else if (even) {
                if (need_w) eg[0] = own[widx];
                if (need_e) eg[3] = own[(size_t)3 * nw + eidx];
            } else {
                if (need_w) eg[0] = own[widx];
                if (need_e) eg[1] = own[(size_t)3 * nw + eidx];
            }
            // row y-1
            if (top) {
                uint64_t v[2][2] = {{0, 0}, {0, 0}}, e = 0;
                // FHP: the edge word is channel 1 west (even rows) or channel 2 east (odd rows)
                const int ek = MODEL == M_HPP ? -1 : (even ? 0 : 1);
                if (!gave_up && !halo_get(halo_slot((unsigned)j, bl, 1), (unsigned)j, ek,
                                          even ? widx : eidx, even ? need_w : need_e, v, e))
                    gave_up = true;
#pragma unroll
                for (int k = 0; k < NV; ++k) {
                    n[0][A0 + k] = v[0][k];
                    n[1][A0 + k] = v[1][k];
                }
                if (MODEL != M_HPP) {
                    if (even) eg[1] = e;
                    else eg[2] = e;
                }
            } else if (active) {
                const uint64_t *up = rows + cur * bufw + (size_t)(r - 1) * roww;
#pragma unroll
                for (int k = 0; k < NV; ++k) {
                    const ulonglong2 v = *reinterpret_cast<const ulonglong2 *>(up + (size_t)(A0 + k) * nw + w0);
                    n[0][A0 + k] = v.x;
                    n[1][A0 + k] = v.y;
                }
                if (MODEL != M_HPP) {
                    if (even && need_w) eg[1] = up[(size_t)1 * nw + widx];
                    if (!even && need_e) eg[2] = up[(size_t)2 * nw + eidx];
                }
            }
            // row y+1
            if (bot) {
                uint64_t v[2][2] = {{0, 0}, {0, 0}}, e = 0;
                // FHP: the edge word is channel 5 west (even rows) or channel 4 east (odd rows)
                const int ek = MODEL == M_HPP ? -1 : (even ? 1 : 0);
                if (!gave_up && !halo_get(halo_slot((unsigned)j, br, 0), (unsigned)j, ek,
                                          even ? widx : eidx, even ? need_w : need_e, v, e))
                    gave_up = true;
#pragma unroll
                for (int k = 0; k < NV; ++k) {
                    n[0][B0 + k] = v[0][k];
                    n[1][B0 + k] = v[1][k];
                }
                if (MODEL != M_HPP) {
                    if (even) eg[2] = e;
                    else eg[3] = e;
                }
            } else if (active) {
                const uint64_t *dn = rows + cur * bufw + (size_t)(r + 1) * roww;
#pragma unroll
                for (int k = 0; k < NV; ++k) {
                    const ulonglong2 v = *reinterpret_cast<const ulonglong2 *>(dn + (size_t)(B0 + k) * nw + w0);
                    n[0][B0 + k] = v.x;
                    n[1][B0 + k] = v.y;
                }
                if (MODEL != M_HPP) {
                    if (even && need_w) eg[2] = dn[(size_t)5 * nw + widx];
                    if (!even && need_e) eg[3] = dn[(size_t)4 * nw + eidx];
                }
            }

            // ---- pull: x-1 / x+1 shifts of the pairs (one shuffle each)
            auto shl = [&](uint64_t v0, uint64_t v1, uint64_t edge, uint64_t &r0, uint64_t &r1) {
                const uint32_t hi = __shfl_up_sync(FULL, (uint32_t)(v1 >> 32), 1);
                const uint64_t in = need_w ? (edge >> 63) : (uint64_t)(hi >> 31);
                r0 = (v0 << 1) | in;
                r1 = (v1 << 1) | (v0 >> 63);
            };
            auto shr = [&](uint64_t v0, uint64_t v1, uint64_t edge, uint64_t &r0, uint64_t &r1) {
                const uint32_t lo = __shfl_down_sync(FULL, (uint32_t)v0, 1);
                const uint64_t in = need_e ? (edge & 1ull) : (uint64_t)(lo & 1u);
                r0 = (v0 >> 1) | (v1 << 63);
                r1 = (v1 >> 1) | (in << 63);
            };
            uint64_t q[2][7];
#pragma unroll
            for (int d = 0; d < D; ++d) {
                q[0][d] = n[0][d];
                q[1][d] = n[1][d];
            }
            if (MODEL == M_HPP) {
                shl(n[0][0], n[1][0], eg[0], q[0][0], q[1][0]);
                shr(n[0][2], n[1][2], eg[1], q[0][2], q[1][2]);
            } else if (even) {  // warp-uniform: one row per warp
                shl(n[0][0], n[1][0], eg[0], q[0][0], q[1][0]);
                shl(n[0][1], n[1][1], eg[1], q[0][1], q[1][1]);
                shl(n[0][5], n[1][5], eg[2], q[0][5], q[1][5]);
                shr(n[0][3], n[1][3], eg[3], q[0][3], q[1][3]);
            } else {
                shl(n[0][0], n[1][0], eg[0], q[0][0], q[1][0]);
                shr(n[0][3], n[1][3], eg[1], q[0][3], q[1][3]);
                shr(n[0][2], n[1][2], eg[2], q[0][2], q[1][2]);
                shr(n[0][4], n[1][4], eg[3], q[0][4], q[1][4]);
            }

            // ---- collision and boundaries (as step_body.cuh), on 32-bit halves
            // of the words: a half's inputs are dead once it is done, which
            // keeps the boundary multiplexer (inputs and outputs live together)
            // within the registers of 28 warps per SM
#pragma unroll
            for (int k = 0; k < 2; ++k) {
                const uint64_t chir = chirality(k);
                const uint64_t ew = (w0 + k == 0 ? 1ull : 0ull) | (w0 + k == nw - 1 ? (1ull << 63) : 0ull);
#pragma unroll
                for (int hf = 0; hf < 2; ++hf) {
                    const int sh = 32 * hf;
                    uint32_t c[7], qh[7];
#pragma unroll
                    for (int d = 0; d < D; ++d) c[d] = qh[d] = (uint32_t)(q[k][d] >> sh);
                    collide_w<MODEL, uint32_t>(c, (uint32_t)(chir >> sh));
                    if (GM != GEOM_NONE && walls) {
                        const uint32_t so = (uint32_t)(solid[k] >> sh), sl = (uint32_t)(slip[k] >> sh);
                        const uint32_t fl = ~(so | sl), e = (uint32_t)(ew >> sh);
#pragma unroll
                        for (int d = 0; d < D; ++d) {
                            uint32_t o = (fl & c[d]) | (so & qh[Dirs<MODEL>::inv(d)]);
                            if (GM == GEOM_FULL) {
                                const uint32_t sx = nsrow ? qh[Dirs<MODEL>::mirx(d)] : qh[d];
                                o |= sl & ((e & qh[Dirs<MODEL>::miry(d)]) | (~e & sx));
                            }
                            c[d] = o;
                        }
                    }
#pragma unroll
                    for (int d = 0; d < D; ++d) {
                        if (hf == 0) s[k][d] = c[d];
                        else s[k][d] |= (uint64_t)c[d] << 32;
                    }
                }
            }

            if (j + 1 < R.nsteps) {
                force(flip_next);
                publish_arrive((unsigned)j + 1);
            }
        }
        if (!RS) {
            if (gave_up && lane == 0) ctl[4 + cur] = 1;
            __syncthreads();
            if (ctl[4 + cur]) return;  // a wait of this step gave up (block-uniform)
        }
    }
    if (RS) {
        if (gave_up && lane == 0) ctl[4] = 1;
        __syncthreads();
        if (ctl[4]) return;  // a wait gave up (block-uniform)
    }

    // the result of the last step: the planes, and the byte-per-cell layout
    // when asked for (after the loop, so that nothing of it stays live there)
    if (active) {
        uint64_t *dp = a.dst + row0 + w0;
#pragma unroll
        for (int d = 0; d < D; ++d)
            *reinterpret_cast<ulonglong2 *>(dp + d * ps) = make_ulonglong2(s[0][d], s[1][d]);
        if (R.aos_out) {
            uint8_t *row = R.aos_out + (size_t)y * (size_t)g.W + (size_t)128 * t;
#pragma unroll
            for (int q = 0; q < 8; ++q) {
                const int k = q >> 2, sh = (q & 3) * 16;
                uint64_t lo = 0, hi = 0;
#pragma unroll
                for (int d = 0; d < D; ++d) {
                    const uint64_t bits = s[k][d] >> sh;
                    lo |= res_spread8(bits & 0xffull) << d;
                    hi |= res_spread8((bits >> 8) & 0xffull) << d;
                }
                reinterpret_cast<uint4 *>(row)[q] =
                    make_uint4((uint32_t)lo, (uint32_t)(lo >> 32), (uint32_t)hi, (uint32_t)(hi >> 32));
            }
        }
    }

    // block sums of the result, fused: each lane counts its words' blocks,
    // the block adds its rows' counts in shared memory (the step buffers are
    // free now), then adds them once per block row and column to the output
    // (a block row can span several bands)
    if (R.sums_B) {
        const int B = R.sums_B, Wb = R.sums_Wb, S = 64 / B;
        // the band's rows again from the block index (nothing kept live for this)
        const int ey0 = (int)((long long)g.H * blockIdx.x / R.nblk);
        const int ey1 = (int)((long long)g.H * (blockIdx.x + 1) / R.nblk);
        const int by0 = ey0 / B, nbr = (ey1 - 1) / B - by0 + 1;
        int *acc = reinterpret_cast<int *>(rows);
        const int nacc = nbr * Wb * 3, nthr = blockDim.x * blockDim.y;
        const int tid = threadIdx.y * blockDim.x + threadIdx.x;
        __syncthreads();  // every warp is done with the step buffers
        for (int i = tid; i < nacc; i += nthr) acc[i] = 0;
        __syncthreads();
        if (active) {
            int *ra = acc + (size_t)(y / B - by0) * Wb * 3;
            for (int k = 0; k < 2; ++k) {
                for (int sb = 0; sb < S; ++sb) {
                    const uint64_t m = (B == 64) ? ~0ull : (((1ull << B) - 1ull) << (sb * B));
                    int n, jx2, jy;
                    res_counts<MODEL>(s[k], m, n, jx2, jy);
                    int *e = ra + (size_t)((w0 + k) * S + sb) * 3;
                    atomicAdd(e, n);
                    atomicAdd(e + 1, jx2);
                    atomicAdd(e + 2, jy);
                }
            }
        }
        __syncthreads();
        for (int i = tid; i < nbr * Wb; i += nthr) {
            const int br = i / Wb, bx = i - br * Wb;
            const size_t o = (size_t)(by0 + br) * Wb + bx;
            atomicAdd(R.sums_N + o, acc[i * 3]);
            atomicAdd(R.sums_Jx2 + o, acc[i * 3 + 1]);
            atomicAdd(R.sums_Jy + o, acc[i * 3 + 2]);
        }
    }
}

#ifndef LGCA_HOST_EMULATION
// ------------------------------------------------------------------ launcher

static size_t resident_smem_bytes(int model, const PlaneGeom &g, int rpb, int wpr)
{
    return res_smem_words(model == M_HPP ? 4 : 6, g.nw, rpb, wpr) * sizeof(uint64_t);
}

bool resident_sums_fit(int model, const PlaneGeom &g, const ResidentShape &sh, int B)
{
    if (!(B == 8 || B == 16 || B == 32 || B == 64)) return false;
    const size_t Wb = (size_t)(g.W + B - 1) / B;
    const size_t nbr = (size_t)(sh.rpb + B - 2) / B + 1;  // block rows a band can touch
    // the accumulators take the step buffers' place
    const size_t bufs = 2 * (size_t)sh.rpb * (model == M_HPP ? 4 : 6) * g.nw * sizeof(uint64_t);
    return nbr * Wb * 3 * sizeof(int) <= bufs;
}

bool resident_shape(int model, const PlaneGeom &g, ResidentShape &out)
{
    if (g.W % 64 != 0 || (g.nw & 1) || g.H < 1) return false;
    const int np = g.nw / 2;
    const int wpr = (np + 31) / 32;
    // the fewest bands of the smallest height the SMs allow: every band has
    // rpb or rpb - 1 rows, and the SMs left over stay free for other streams'
    // kernels (e.g. the layout conversions of an upload or a download, which
    // then overlap the steps)
    const int rpb = (g.H + std::min(sm_count(), g.H) - 1) / std::min(sm_count(), g.H);
    const int nblk = (g.H + rpb - 1) / rpb;
    if (rpb * wpr > RES_MAX_WARPS) return false;
    const size_t smem = resident_smem_bytes(model, g, rpb, wpr);
    if (smem > RES_MAX_SMEM) return false;
    out.nblk = nblk;
    out.wpr = wpr;
    out.rpb = rpb;
    out.smem = smem;
    out.rowsync = model >= M_FHP_II && rpb * wpr >= RES_ROWSYNC_WARPS;
    out.halo_words = (size_t)RES_HALO_SLOTS * nblk * 2 * 2 * g.nw * 2;
    return true;
}

template <int MODEL, int GM, bool RS>
static cudaError_t res_launch(const StepArgs &a, const ResidentShape &sh, const ResidentArgs &R,
                              cudaStream_t st)
{
    auto kern = k_resident<MODEL, GM, RS>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sh.smem);
    if (e != cudaSuccess) return e;
    int per_sm = 0;
    const int threads = 32 * sh.rpb * sh.wpr;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, sh.smem);
    if (e != cudaSuccess) return e;
    if (per_sm < 1 || sh.nblk > per_sm * sm_count()) return cudaErrorCooperativeLaunchTooLarge;
    StepArgs aa = a;
    ResidentArgs rr = R;
    void *args[] = {(void *)&aa, (void *)&rr};
    return cudaLaunchCooperativeKernel((void *)kern, dim3(sh.nblk), dim3(32, sh.rpb * sh.wpr), args,
                                      sh.smem, st);
}

template <int MODEL, bool RS>
static cudaError_t res_model(int gm, const StepArgs &a, const ResidentShape &sh,
                             const ResidentArgs &R, cudaStream_t st)
{
    switch (gm) {
    case GEOM_NONE: return res_launch<MODEL, GEOM_NONE, RS>(a, sh, R, st);
    case GEOM_NOSLIP: return res_launch<MODEL, GEOM_NOSLIP, RS>(a, sh, R, st);
    default: return res_launch<MODEL, GEOM_FULL, RS>(a, sh, R, st);
    }
}

cudaError_t launch_resident(int model, int gm, const StepArgs &a, const ResidentShape &sh,
                            uint64_t *halo, int *err, uint64_t seed, uint64_t t0,
                            int nsteps, const PersistWait &w, const uint8_t *aos_in,
                            uint8_t *aos_out, const ResidentSums *sums, unsigned epoch,
                            cudaStream_t st)
{
    if (w.wait_ns == 0 || nsteps < 1 || nsteps > RESIDENT_MAX_STEPS || epoch < 1 || epoch > 255)
        return cudaErrorInvalidValue;
    ResidentArgs R;
    R.halo = halo;
    R.epoch = epoch;
    R.err = err;
    R.seed = seed;
    R.t0 = t0;
    R.nsteps = nsteps;
    R.nblk = sh.nblk;
    R.wpr = sh.wpr;
    R.rpb = sh.rpb;
    R.wait_ns = w.wait_ns;
    R.withhold = w.withhold;
    R.aos_in = aos_in;
    R.aos_out = aos_out;
    R.sums_B = sums ? sums->B : 0;
    R.sums_Wb = sums ? (a.g.W + sums->B - 1) / sums->B : 0;
    R.sums_N = sums ? sums->N : nullptr;
    R.sums_Jx2 = sums ? sums->Jx2 : nullptr;
    R.sums_Jy = sums ? sums->Jy : nullptr;
    // row barriers for FHP-II/III blocks of many warps (measured on GB300:
    // 1-3.5 % faster there; slower for HPP and FHP-I, and on blocks of 14
    // warps)
    switch (model) {
    case M_HPP: return res_model<M_HPP, false>(gm, a, sh, R, st);
    case M_FHP_I: return res_model<M_FHP_I, false>(gm, a, sh, R, st);
    default:  // FHP-II and FHP-III share one rule set
        return sh.rowsync ? res_model<M_FHP_II, true>(gm, a, sh, R, st)
                          : res_model<M_FHP_II, false>(gm, a, sh, R, st);
    }
}
#endif

}  // namespace lgca_gpu
