// Plain lattice step (one step per pass over global memory).
//
// Reference: OMP_Lattice<M>::collide_and_propagate, keva92/lgca
// src/omp_lattice.cpp:100-249.  The reference pulls, for every cell and
// channel d, the bit of channel d of the cell at offset_to_neighbor[INV_DIR[d]]
// plus the periodic edge corrections (src/lgca_models.h:79-132 HPP,
// :292-365 / :483-566 / :701-784 FHP).  With an even number of rows those
// tables describe a torus; the source cell of channel d of site (x, y) is
//
//   d   FHP, y even   FHP, y odd    HPP
//   0   (x-1, y)      (x-1, y)      (x-1, y)
//   1   (x-1, y-1)    (x,   y-1)    (x,   y-1)
//   2   (x,   y-1)    (x+1, y-1)    (x+1, y)
//   3   (x+1, y)      (x+1, y)      (x,   y+1)
//   4   (x,   y+1)    (x+1, y+1)
//   5   (x-1, y+1)    (x,   y+1)
//   6   (x,   y)      (x,   y)
//
// all coordinates modulo (W, H).  On bit-planes every channel is read from a
// single row, and an x offset of +-1 is a one-bit shift of the word with the
// missing bit taken from the neighbouring word (a warp shuffle, or a load at
// a warp edge / the periodic x seam).
//
// Mapping (set by the caller): each lane holds one word (step_word) or two
// words (step_pair) of one row; consecutive lanes hold consecutive words of
// a row, and a lane whose neighbour lane holds another row (or no row) loads
// the neighbour word instead of shuffling.  Each lane loads D words (or
// pairs) and stores as many; the only other traffic is one word per shifted
// plane at row and warp edges.
#pragma once
#include "internal.cuh"
#include "../../include/lgca/rng.h"

namespace lgca_gpu {

static constexpr unsigned FULL = 0xffffffffu;

// What changes from one step to the next: the two buffers and the keys.
struct StepIO {
    const uint64_t *__restrict__ src;
    uint64_t *__restrict__ dst;
    uint64_t ckey, fkey;  // chirality / forcing keys of the step
};

// State loads: CG = ld.global.cg, cached in L2 only, for kernels whose input
// was written while they (or a kernel overlapping them on the same SMs) were
// resident -- the persistent band kernel, and the step kernels chained by
// programmatic dependent launch; otherwise the read-only path.
template <bool CG> __device__ __forceinline__ uint64_t ld_state(const uint64_t *p)
{
    return CG ? __ldcg(p) : __ldg(p);
}
template <bool CG> __device__ __forceinline__ ulonglong2 ld_state2(const uint64_t *p)
{
    return CG ? __ldcg(reinterpret_cast<const ulonglong2 *>(p))
              : __ldg(reinterpret_cast<const ulonglong2 *>(p));
}

// Forcing decision at site (fx, y): a FLUID cell with channel 0 empty and the
// west-moving channel (3 for FHP, 2 for HPP) occupied reverses with
// probability thr / 2^32.  Used by the lanes that fetch the forced word from
// another chunk.
template <int MODEL, int GM, bool CG = false>
__device__ __forceinline__ uint64_t force_flip_at(const StepArgs &a, const StepIO &io, int y)
{
    constexpr int WEST = (MODEL == M_HPP) ? 2 : 3;
    const int fw = a.fx >> 6, fb = a.fx & 63;
    const unsigned r0 = (unsigned)y * a.g.pitch + fw;
    uint64_t n0 = ld_state<CG>(io.src + r0), nw = ld_state<CG>(io.src + (WEST * (unsigned)a.g.ps + r0));
    uint64_t fluid = ~0ull;
    if (GM >= GEOM_NOSLIP) fluid &= ~a.solid[r0];
    if (GM == GEOM_FULL) fluid &= ~a.slip[r0];
    const uint64_t u = lgca_rng_draw(io.fkey, lgca_rng_index((uint32_t)y, (uint32_t)a.fx)) >> 32;
    const uint64_t cand = (~n0 & nw & fluid) >> fb & 1ull;
    return (u < a.force_thr) ? cand : 0ull;
}

// Row mapping contract of both step bodies: the lanes of a warp hold rows of
// one parity (FHP shifts depend on it, and the shuffles must be executed by
// the whole warp), e.g. rows y, y+2, ... when rows are narrower than a warp.
// `pre` carries chirality words drawn before the caller waited for the
// previous step (PRE); they equal lgca_rng_draw(io.ckey, (y, word)).
template <int MODEL, int GM, bool CG = false, bool PRE = false>
__device__ __forceinline__ void step_word(const StepArgs &a, const StepIO &io, const int y,
                                          const int w, const int lane, const int width = 32,
                                          const uint64_t pre = 0)
{
    constexpr int D = ModelTraits<MODEL>::D;
    const PlaneGeom &g = a.g;
    const bool active = w < g.nw && y < g.H;
    const int seg = lane & (width - 1);  // lane within its row segment
    const int ym = (y == 0) ? g.H - 1 : y - 1;
    const int yp = (y == g.H - 1) ? 0 : y + 1;
    // 32-bit offsets: a lattice has at most 2^31 sites, so D * H * pitch < 2^29 words
    const unsigned rowm = (unsigned)ym * g.pitch, row0 = (unsigned)y * g.pitch,
                   rowp = (unsigned)yp * g.pitch;
    const uint64_t *__restrict__ s = io.src;
    const unsigned ps = (unsigned)g.ps;
    const bool even = (y & 1) == 0;

    // which plane comes from which row (see the table above)
    // HPP: 0 -> row y, 1 -> row y-1, 2 -> row y, 3 -> row y+1
    // FHP: 0,3,6 -> row y, 1,2 -> row y-1, 4,5 -> row y+1
    auto row_of = [&](int d) -> unsigned {
        if (MODEL == M_HPP) return d == 1 ? rowm : (d == 3 ? rowp : row0);
        return (d == 1 || d == 2) ? rowm : ((d == 4 || d == 5) ? rowp : row0);
    };

    uint64_t n[7];
#pragma unroll
    for (int d = 0; d < D; ++d) n[d] = active ? ld_state<CG>(s + (d * ps + row_of(d) + w)) : 0ull;

    uint64_t solid = 0, slip = 0;
    if (GM >= GEOM_NOSLIP && active) solid = __ldg(a.solid + row0 + w);
    if (GM == GEOM_FULL && active) slip = __ldg(a.slip + row0 + w);

    // forcing column: applied to the source words before the pull
    constexpr int WEST = (MODEL == M_HPP) ? 2 : 3;
    const bool forcing = a.force_thr != 0;
    if (forcing && active && w == (a.fx >> 6)) {
        const int fb = a.fx & 63;
        const uint64_t u =
            lgca_rng_draw(io.fkey, lgca_rng_index((uint32_t)y, (uint32_t)a.fx)) >> 32;
        const uint64_t fl = (u < a.force_thr) ? ((~n[0] & n[WEST] & ~solid & ~slip) >> fb & 1ull) : 0ull;
        n[0] |= fl << fb;
        n[WEST] &= ~(fl << fb);
    }

    // neighbour words at row and warp edges and the periodic x seam, one per
    // shifted plane (see step_pair for the planes per model and parity)
    const bool need_w = active && (seg == 0 || w == 0);
    const bool need_e = active && (seg == width - 1 || w == g.nw - 1);
    const int widx = (w == 0) ? g.nw - 1 : w - 1;
    const int wbit = (w == 0) ? g.L : 63;
    const int eidx = (w == g.nw - 1) ? 0 : w + 1;
    const int epos = (w == g.nw - 1) ? g.L : 63;
    const int wx = (w == 0) ? g.W - 1 : 64 * w - 1;  // site of the fetched west bit
    const int ex = (w == g.nw - 1) ? 0 : 64 * w + 64; // site of the fetched east bit
    auto ldw = [&](int d, unsigned row) -> uint64_t { return ld_state<CG>(s + (d * ps + row + widx)); };
    auto lde = [&](int d, unsigned row) -> uint64_t { return ld_state<CG>(s + (d * ps + row + eidx)); };
    uint64_t eg[4] = {0, 0, 0, 0};
    if (MODEL == M_HPP) {
        if (need_w) eg[0] = ldw(0, row0);
        if (need_e) eg[1] = lde(2, row0);
    } else if (even) {
        if (need_w) {
            eg[0] = ldw(0, row0);
            eg[1] = ldw(1, rowm);
            eg[2] = ldw(5, rowp);
        }
        if (need_e) eg[3] = lde(3, row0);
    } else {
        if (need_w) eg[0] = ldw(0, row0);
        if (need_e) {
            eg[1] = lde(3, row0);
            eg[2] = lde(2, rowm);
            eg[3] = lde(4, rowp);
        }
    }

    // x-1 pull: (v << 1) | bit of site x-1 (from `edge` in lanes with need_w)
    auto shl = [&](uint64_t v, uint64_t edge, bool fcol) -> uint64_t {
        const uint32_t hi = __shfl_up_sync(FULL, (uint32_t)(v >> 32), 1, width);
        uint64_t in = hi >> 31;
        if (need_w) {
            in = (edge >> wbit) & 1ull;
            if (fcol && forcing && wx == a.fx) in |= force_flip_at<MODEL, GM, CG>(a, io, y);
        }
        return (v << 1) | in;
    };
    // x+1 pull: (v >> 1) | bit of site x+1 placed at the last valid bit
    auto shr = [&](uint64_t v, uint64_t edge, bool fcol) -> uint64_t {
        const uint32_t lo = __shfl_down_sync(FULL, (uint32_t)v, 1, width);
        uint64_t in = lo & 1u;
        if (need_e) {
            in = edge & 1ull;
            if (fcol && forcing && ex == a.fx) in &= ~force_flip_at<MODEL, GM, CG>(a, io, y);
        }
        return (v >> 1) | (in << epos);
    };

    uint64_t p[7];
    if (MODEL == M_HPP) {
        p[0] = shl(n[0], eg[0], true);
        p[1] = n[1];
        p[2] = shr(n[2], eg[1], true);
        p[3] = n[3];
    } else if (even) {  // warp-uniform (row mapping contract)
        p[0] = shl(n[0], eg[0], true);
        p[1] = shl(n[1], eg[1], false);
        p[5] = shl(n[5], eg[2], false);
        p[3] = shr(n[3], eg[3], true);
        p[2] = n[2];
        p[4] = n[4];
        if (D == 7) p[6] = n[6];
    } else {
        p[0] = shl(n[0], eg[0], true);
        p[3] = shr(n[3], eg[1], true);
        p[2] = shr(n[2], eg[2], false);
        p[4] = shr(n[4], eg[3], false);
        p[1] = n[1];
        p[5] = n[5];
        if (D == 7) p[6] = n[6];
    }
    // warps without wall or obstacle cells skip the boundary multiplexer (a
    // vote of all lanes, before the inactive ones leave)
    const bool walls = GM != GEOM_NONE && __any_sync(FULL, (solid | slip) != 0ull);
    if (!active) return;

    uint64_t c[7];
#pragma unroll
    for (int d = 0; d < D; ++d) c[d] = p[d];
    if (MODEL != M_HPP) {
        const uint64_t chir =
            a.chir ? __ldg(a.chir + row0 + w)
                   : (PRE ? pre : lgca_rng_draw(io.ckey, lgca_rng_index((uint32_t)y, (uint32_t)w)));
        collide<MODEL>(c, chir);
    } else {
        collide<MODEL>(c, 0ull);
    }

    uint64_t out[7];
    if (GM == GEOM_NONE || !walls) {
#pragma unroll
        for (int d = 0; d < D; ++d) out[d] = c[d];
    } else {
        const uint64_t fluid = ~(solid | slip);
        // slip cells: mirror in x on the first/last row, in y on the first/last
        // column (the latter wins at corners), unchanged elsewhere
        const bool nsrow = (y == 0) || (y == g.H - 1);
        const uint64_t ew = (w == 0 ? 1ull : 0ull) | (w == g.nw - 1 ? (1ull << g.L) : 0ull);
#pragma unroll
        for (int d = 0; d < D; ++d) {
            uint64_t o = (fluid & c[d]) | (solid & p[Dirs<MODEL>::inv(d)]);
            if (GM == GEOM_FULL) {
                const uint64_t sx = nsrow ? p[Dirs<MODEL>::mirx(d)] : p[d];
                const uint64_t sl = (ew & p[Dirs<MODEL>::miry(d)]) | (~ew & sx);
                o |= slip & sl;
            }
            out[d] = o;
        }
    }
    if (w == g.nw - 1) {  // clear the tail bits past site W-1
#pragma unroll
        for (int d = 0; d < D; ++d) out[d] &= g.lastmask;
    }
    uint64_t *__restrict__ dp = io.dst + row0 + w;
#pragma unroll
    for (int d = 0; d < D; ++d) dp[d * ps] = out[d];
}

// Two words per lane (lattices with an even number of words per row, i.e.
// W a multiple of 64): 16-byte loads and stores, one shuffle per shifted
// plane for 128 sites, and half as many warps, so that an L2-resident lattice
// fits in one wave of resident warps.  Same arithmetic as step_word.  With an
// odd number of words per row (ODD) the last pair holds the last word and the
// row's padding word (the pitch is even): that word's east neighbour is the
// seam word, and the padding word is written back as zero.  With WRAP the
// periodic seam words of a row that lies inside the lane segment come from
// the row's own first and last lanes by shuffle, so that narrow rows (a few
// lane items each) load no edge words at all; only words held by another
// segment are loaded.
template <int MODEL, int GM, bool CG = false, bool PRE = false, bool ODD = false,
          bool WRAP = false>
__device__ __forceinline__ void step_pair(const StepArgs &a, const StepIO &io, const int y,
                                          const int t, const int lane, const int width = 32,
                                          const uint64_t pre0 = 0, const uint64_t pre1 = 0)
{
    constexpr int D = ModelTraits<MODEL>::D;
    const PlaneGeom &g = a.g;
    const int np = (g.nw + 1) >> 1;
    const bool active = t < np && y < g.H;
    const bool half = ODD && t == np - 1;  // (ODD: odd words per row) the second word is padding
    const int seg = lane & (width - 1);  // lane within its row segment
    const int ym = (y == 0) ? g.H - 1 : y - 1;
    const int yp = (y == g.H - 1) ? 0 : y + 1;
    const unsigned rowm = (unsigned)ym * g.pitch, row0 = (unsigned)y * g.pitch,
                   rowp = (unsigned)yp * g.pitch;
    const uint64_t *__restrict__ s = io.src;
    const unsigned ps = (unsigned)g.ps;
    const bool even = (y & 1) == 0;
    const int w0 = 2 * t;
    auto row_of = [&](int d) -> unsigned {
        if (MODEL == M_HPP) return d == 1 ? rowm : (d == 3 ? rowp : row0);
        return (d == 1 || d == 2) ? rowm : ((d == 4 || d == 5) ? rowp : row0);
    };
    auto ld2 = [&](const uint64_t *base, unsigned off) -> ulonglong2 {  // state
        return active ? ld_state2<CG>(base + off) : make_ulonglong2(0ull, 0ull);
    };
    auto ldg2 = [&](const uint64_t *base, unsigned off) -> ulonglong2 {  // read-only planes
        return active ? __ldg(reinterpret_cast<const ulonglong2 *>(base + off))
                      : make_ulonglong2(0ull, 0ull);
    };

    uint64_t n[2][7];
#pragma unroll
    for (int d = 0; d < D; ++d) {
        const ulonglong2 v = ld2(s, d * ps + row_of(d) + w0);
        n[0][d] = v.x;
        n[1][d] = v.y;
    }
    uint64_t solid[2] = {0, 0}, slip[2] = {0, 0};
    if (GM >= GEOM_NOSLIP) {
        const ulonglong2 v = ldg2(a.solid, row0 + w0);
        solid[0] = v.x;
        solid[1] = v.y;
    }
    if (GM == GEOM_FULL) {
        const ulonglong2 v = ldg2(a.slip, row0 + w0);
        slip[0] = v.x;
        slip[1] = v.y;
    }

    // Edge words, loaded with the state so that their latency overlaps it:
    // a lane whose left (right) neighbour lane holds another row, or none,
    // takes the word west (east) of its pair from memory for every plane that
    // shifts that way.  Which planes shift which way depends on the model
    // and the row parity (warp-uniform):
    //   FHP, even row: west 0 (row y), 1 (y-1), 5 (y+1); east 3 (row y)
    //   FHP, odd row:  west 0 (row y); east 3 (row y), 2 (y-1), 4 (y+1)
    //   HPP:           west 0 (row y); east 2 (row y)
    // source lanes, within the segment, of the words west and east of the
    // pair: the neighbouring items of the row, or across the seam (WRAP) the
    // row's last / first item; a source outside the segment means a load
    const int srcw = WRAP ? seg + (t == 0 ? np - 1 : -1) : seg - 1;
    const int srce = WRAP ? seg + (t == np - 1 ? 1 - np : 1) : seg + 1;
    const bool need_w =
        active && (WRAP ? (unsigned)srcw >= (unsigned)width : (seg == 0 || t == 0));
    const bool need_e =
        active && (WRAP ? (unsigned)srce >= (unsigned)width : (seg == width - 1 || t == np - 1));
    const int widx = (t == 0) ? g.nw - 1 : w0 - 1;
    const int eidx = (t == np - 1) ? 0 : w0 + 2;
    auto ldw = [&](int d, unsigned row) -> uint64_t { return ld_state<CG>(s + (d * ps + row + widx)); };
    auto lde = [&](int d, unsigned row) -> uint64_t { return ld_state<CG>(s + (d * ps + row + eidx)); };
    uint64_t eg[4] = {0, 0, 0, 0};  // in the order the pulls below use them
    if (MODEL == M_HPP) {
        if (need_w) eg[0] = ldw(0, row0);
        if (need_e) eg[1] = lde(2, row0);
    } else if (even) {
        if (need_w) {
            eg[0] = ldw(0, row0);
            eg[1] = ldw(1, rowm);
            eg[2] = ldw(5, rowp);
        }
        if (need_e) eg[3] = lde(3, row0);
    } else {
        if (need_w) eg[0] = ldw(0, row0);
        if (need_e) {
            eg[1] = lde(3, row0);
            eg[2] = lde(2, rowm);
            eg[3] = lde(4, rowp);
        }
    }

    constexpr int WEST = (MODEL == M_HPP) ? 2 : 3;
    const bool forcing = a.force_thr != 0;
    const int fw = a.fx >> 6;
    if (forcing && active && (fw >> 1) == t) {
        const uint64_t u =
            lgca_rng_draw(io.fkey, lgca_rng_index((uint32_t)y, (uint32_t)a.fx)) >> 32;
        const uint64_t bit = (u < a.force_thr) ? (1ull << (a.fx & 63)) : 0ull;
        // masks per word of the pair (no run-time index into n, which would
        // move the arrays to local memory)
        const uint64_t m0 = (fw & 1) ? 0ull : bit, m1 = (fw & 1) ? bit : 0ull;
        const uint64_t f0 = ~n[0][0] & n[0][WEST] & ~solid[0] & ~slip[0] & m0;
        const uint64_t f1 = ~n[1][0] & n[1][WEST] & ~solid[1] & ~slip[1] & m1;
        n[0][0] |= f0;
        n[0][WEST] &= ~f0;
        n[1][0] |= f1;
        n[1][WEST] &= ~f1;
    }

    const int wx = (t == 0) ? g.W - 1 : 64 * w0 - 1;
    const int ex = (t == np - 1) ? 0 : 64 * w0 + 128;

    // x-1 pull of the pair (v0, v1) into (r0, r1); `edge` is the word west of
    // it, read by lanes with need_w (and forced there when it holds the
    // forcing column).  One shuffle per pair: only the first word takes a bit
    // from outside the pair.
    auto shl = [&](uint64_t v0, uint64_t v1, uint64_t edge, bool fcol, uint64_t &r0, uint64_t &r1) {
        // a lane offers the high half of its last real word (v0 in a half pair)
        const uint32_t hi =
            WRAP ? __shfl_sync(FULL, (uint32_t)((half ? v0 : v1) >> 32), srcw, width)
                 : __shfl_up_sync(FULL, (uint32_t)(v1 >> 32), 1, width);
        uint64_t in = hi >> 31;
        if (need_w) {
            in = edge >> 63;
            if (fcol && forcing && wx == a.fx) in |= force_flip_at<MODEL, GM, CG>(a, io, y);
        }
        r0 = (v0 << 1) | in;
        r1 = (v1 << 1) | (v0 >> 63);
    };
    // x+1 pull of the pair into (r0, r1); `edge` is the word east of it
    auto shr = [&](uint64_t v0, uint64_t v1, uint64_t edge, bool fcol, uint64_t &r0, uint64_t &r1) {
        const uint32_t lo = WRAP ? __shfl_sync(FULL, (uint32_t)v0, srce, width)
                                 : __shfl_down_sync(FULL, (uint32_t)v0, 1, width);
        uint64_t in = lo & 1u;
        if (need_e) {
            in = edge & 1ull;
            if (fcol && forcing && ex == a.fx) in &= ~force_flip_at<MODEL, GM, CG>(a, io, y);
        }
        r0 = (v0 >> 1) | ((half ? in : v1) << 63);
        r1 = (v1 >> 1) | (in << 63);
    };
    // pulled values of word k of the pair
    uint64_t q[2][7];
    if (MODEL == M_HPP) {
        shl(n[0][0], n[1][0], eg[0], true, q[0][0], q[1][0]);
        shr(n[0][2], n[1][2], eg[1], true, q[0][2], q[1][2]);
        q[0][1] = n[0][1]; q[1][1] = n[1][1]; q[0][3] = n[0][3]; q[1][3] = n[1][3];
    } else if (even) {  // warp-uniform (row mapping contract)
        shl(n[0][0], n[1][0], eg[0], true, q[0][0], q[1][0]);
        shl(n[0][1], n[1][1], eg[1], false, q[0][1], q[1][1]);
        shl(n[0][5], n[1][5], eg[2], false, q[0][5], q[1][5]);
        shr(n[0][3], n[1][3], eg[3], true, q[0][3], q[1][3]);
        q[0][2] = n[0][2]; q[1][2] = n[1][2]; q[0][4] = n[0][4]; q[1][4] = n[1][4];
        if (D == 7) { q[0][6] = n[0][6]; q[1][6] = n[1][6]; }
    } else {
        shl(n[0][0], n[1][0], eg[0], true, q[0][0], q[1][0]);
        shr(n[0][3], n[1][3], eg[1], true, q[0][3], q[1][3]);
        shr(n[0][2], n[1][2], eg[2], false, q[0][2], q[1][2]);
        shr(n[0][4], n[1][4], eg[3], false, q[0][4], q[1][4]);
        q[0][1] = n[0][1]; q[1][1] = n[1][1]; q[0][5] = n[0][5]; q[1][5] = n[1][5];
        if (D == 7) { q[0][6] = n[0][6]; q[1][6] = n[1][6]; }
    }
    // whether any lane of the warp holds a wall or obstacle cell (a vote of
    // all lanes, before the inactive ones leave): warps without one skip the
    // boundary multiplexer
    const bool walls = GM != GEOM_NONE &&
                       __any_sync(FULL, (solid[0] | solid[1] | slip[0] | slip[1]) != 0ull);
    if (!active) return;

    const bool nsrow = (y == 0) || (y == g.H - 1);
    uint64_t out[2][7];
#pragma unroll
    for (int k = 0; k < 2; ++k) {
        uint64_t p[7], c[7];
#pragma unroll
        for (int d = 0; d < D; ++d) c[d] = p[d] = q[k][d];
        if (MODEL != M_HPP) {
            const uint64_t chir =
                a.chir ? __ldg(a.chir + row0 + w0 + k)
                       : (PRE ? (k ? pre1 : pre0)
                              : lgca_rng_draw(io.ckey, lgca_rng_index((uint32_t)y, (uint32_t)(w0 + k))));
            collide<MODEL>(c, chir);
        } else {
            collide<MODEL>(c, 0ull);
        }
        if (GM == GEOM_NONE || !walls) {
#pragma unroll
            for (int d = 0; d < D; ++d) out[k][d] = c[d];
        } else {
            const uint64_t fl = ~(solid[k] | slip[k]);
            const uint64_t ew = (w0 + k == 0 ? 1ull : 0ull) | (w0 + k == g.nw - 1 ? (1ull << 63) : 0ull);
#pragma unroll
            for (int d = 0; d < D; ++d) {
                uint64_t o = (fl & c[d]) | (solid[k] & p[Dirs<MODEL>::inv(d)]);
                if (GM == GEOM_FULL) {
                    const uint64_t sx = nsrow ? p[Dirs<MODEL>::mirx(d)] : p[d];
                    o |= slip[k] & ((ew & p[Dirs<MODEL>::miry(d)]) | (~ew & sx));
                }
                out[k][d] = o;
            }
        }
    }
    uint64_t *__restrict__ dp = io.dst + row0 + w0;
#pragma unroll
    for (int d = 0; d < D; ++d)
        *reinterpret_cast<ulonglong2 *>(dp + d * ps) =
            make_ulonglong2(out[0][d], half ? 0ull : out[1][d]);
}

}  // namespace lgca_gpu
