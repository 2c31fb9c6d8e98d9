// Host emulation of the batched step (lgca_gb300/csrc/batch_kernels.cuh:
// k_batch_keys, k_batch and k_batch_wave) for CPU parity checks of the batch
// kernel code.
// The kernels are compiled here as plain C++ by g++ and run on the grids the
// launchers use: a pool of 256 host threads plays one block at a time, a warp
// shuffle is an exchange among a warp's 32 threads between two barrier
// waits.  The call's work-list (entries sorted by steps, then by kernel
// code; each member's warp tasks padded to whole blocks; the block -> member
// map; segments of constant active sets with the step counter; members on
// the register wavefront with their single steps in the one-step list and
// their passes in a list per depth) is restated from lgca_batch_step_each
// (lgca_gb300/csrc/lgca_gpu.cu).  tests/test_step_emulated.py compares every
// member with the oracle.
//
//   batch_emu IN OUT
//   IN:  int32 members, warp_tasks; then per member: int32 model, W, H,
//        nsteps, force_x, depth (0 or 1: one step per launch; 2, 4, 8: the
//        wavefront where it applies); uint64 seed, t0, force_thr; H*W uint8
//        cells; H*W uint8 cell types (0 fluid, 1 no-slip, 2 slip)
//   OUT: per member, H*W uint8 cells after its steps
#include <algorithm>
#include <cstdint>
#include <cstdlib>
#include <cstdio>
#include <cstring>
#include <functional>

#include <barrier>
#include <thread>
#include <vector>

#include <cuda_runtime.h>

namespace emu {
struct Warp {
    uint32_t v[32];
    std::barrier<> bar{32};
};
thread_local int lane = 0;
thread_local Warp *warp = nullptr;

inline uint32_t exchange(uint32_t v, int src)
{
    warp->v[lane] = v;
    warp->bar.arrive_and_wait();
    const uint32_t r = warp->v[src];
    warp->bar.arrive_and_wait();
    return r;
}
}  // namespace emu

thread_local uint3 threadIdx;
thread_local uint3 blockIdx;
thread_local dim3 blockDim;
thread_local dim3 gridDim;  // (only the persistent kernel, not run here, reads it)

inline uint32_t __shfl_sync(unsigned, uint32_t v, int src, int width = 32)
{
    const int base = emu::lane & ~(width - 1);
    return emu::exchange(v, base + (src & (width - 1)));
}
inline uint32_t __shfl_up_sync(unsigned, uint32_t v, unsigned delta, int width = 32)
{
    const int base = emu::lane & ~(width - 1);
    const int s = emu::lane - (int)delta;
    return emu::exchange(v, s < base ? emu::lane : s);
}
inline uint32_t __shfl_down_sync(unsigned, uint32_t v, unsigned delta, int width = 32)
{
    const int base = emu::lane & ~(width - 1);
    const int s = emu::lane + (int)delta;
    return emu::exchange(v, s >= base + width ? emu::lane : s);
}
// warp vote: every lane offers its predicate, each gets the OR of all
inline int __any_sync(unsigned, int pred)
{
    emu::warp->v[emu::lane] = pred != 0;
    emu::warp->bar.arrive_and_wait();
    int any = 0;
    for (int i = 0; i < 32; ++i) any |= (int)emu::warp->v[i];
    emu::warp->bar.arrive_and_wait();
    return any;
}
// used only by the persistent batch kernel, which is compiled here but not run
inline void __syncthreads() { std::abort(); }
inline void __nanosleep(unsigned) { std::abort(); }
inline void __threadfence() { std::abort(); }
inline int atomicExch(int *, int) { std::abort(); }
inline unsigned atomicAdd(unsigned *, unsigned) { std::abort(); }
template <class T> inline T __ldcg(const T *p) { return *p; }
template <class T> inline T __ldg(const T *p) { return *p; }
#ifndef __launch_bounds__
#define __launch_bounds__(...)
#endif
#ifndef __grid_constant__
#define __grid_constant__
#endif

#include "../lgca_gb300/csrc/batch_kernels.cuh"

using namespace lgca_gpu;

// a grid of `blocks` blocks of `threads` threads, one block at a time
static void run_grid(unsigned blocks, const std::function<void()> &body, int threads = 256)
{
    if (blocks == 0) return;
    std::vector<emu::Warp> warps(threads / 32);
    std::barrier<> done(threads);
    std::vector<std::thread> th;
    for (int i = 0; i < threads; ++i)
        th.emplace_back([&, i] {
            threadIdx = make_uint3((unsigned)i, 0, 0);
            blockDim = dim3((unsigned)threads, 1, 1);
            emu::lane = i & 31;
            emu::warp = &warps[i >> 5];
            for (unsigned b = 0; b < blocks; ++b) {
                blockIdx = make_uint3(b, 0, 0);
                body();
                done.arrive_and_wait();  // the block is complete before the next starts
            }
        });
    for (auto &x : th) x.join();
}

struct Member {
    int model, W, H, nsteps, fx, K;
    uint64_t seed, t0, thr;
    std::vector<uint8_t> cells, types;
    PlaneGeom g;
    std::vector<uint64_t> buf[2], solid, slip;
    int cur = 0, gm = GEOM_NONE;
};

int main(int argc, char **argv)
{
    if (argc != 3) {
        std::fprintf(stderr, "usage: batch_emu IN OUT\n");
        return 2;
    }
    FILE *f = std::fopen(argv[1], "rb");
    if (!f) return 2;
    int32_t top[2];
    if (std::fread(top, sizeof(top), 1, f) != 1) return 2;
    const int nm = top[0], wt = top[1];
    if (!(wt == 1 || wt == 2 || wt == 4 || wt == 8)) return 3;
    std::vector<Member> M(nm);
    for (auto &m : M) {
        int32_t h[6];
        uint64_t u[3];
        if (std::fread(h, sizeof(h), 1, f) != 1 || std::fread(u, sizeof(u), 1, f) != 1) return 2;
        m.model = h[0], m.W = h[1], m.H = h[2], m.nsteps = h[3], m.fx = h[4], m.K = h[5];
        m.seed = u[0], m.t0 = u[1], m.thr = u[2];
        m.cells.resize((size_t)m.W * m.H);
        m.types.resize((size_t)m.W * m.H);
        if (std::fread(m.cells.data(), 1, m.cells.size(), f) != m.cells.size() ||
            std::fread(m.types.data(), 1, m.types.size(), f) != m.types.size())
            return 2;
        PlaneGeom &g = m.g;
        g.W = m.W;
        g.H = m.H;
        g.nw = (m.W + 63) / 64;
        g.pitch = (g.nw + 1) & ~1;
        g.ps = (size_t)m.H * g.pitch;
        g.L = (m.W - 1) & 63;
        g.lastmask = (g.L == 63) ? ~0ull : ((1ull << (g.L + 1)) - 1ull);
        const int D = num_dir(m.model);
        m.buf[0].assign(D * g.ps, 0);
        m.buf[1].assign(D * g.ps, 0);
        m.solid.assign(g.ps, 0);
        m.slip.assign(g.ps, 0);
        bool any_solid = false, any_slip = false;
        for (int y = 0; y < m.H; ++y)
            for (int x = 0; x < m.W; ++x) {
                const size_t o = (size_t)y * g.pitch + (x >> 6);
                const uint64_t bit = 1ull << (x & 63);
                const uint8_t c = m.cells[(size_t)y * m.W + x];
                for (int d = 0; d < D; ++d)
                    if ((c >> d) & 1) m.buf[0][d * g.ps + o] |= bit;
                const uint8_t ty = m.types[(size_t)y * m.W + x];
                if (ty == 1) m.solid[o] |= bit, any_solid = true;
                if (ty == 2) m.slip[o] |= bit, any_slip = true;
            }
        m.gm = any_slip ? GEOM_FULL : (any_solid ? GEOM_NOSLIP : GEOM_NONE);
    }
    std::fclose(f);

    // ---- the work-lists of one call (lgca_batch_step_each)
    // depth of a member on the wavefront (wave_depth), 0 for one step per launch
    for (auto &m : M) {
        const bool ok = (m.K == 2 || m.K == 4 || (m.K == 8 && m.model == 0)) && m.W % 64 == 0 &&
                        m.H >= 2 && m.nsteps >= m.K;
        if (!ok) m.K = 0;
    }
    auto singles = [](const Member &m) { return m.K ? m.nsteps % m.K : m.nsteps; };
    auto pair_of = [](const Member &m) { return (m.W % 64) == 0; };
    auto code_of = [&](const Member &m) {
        const int fam = m.model == 0 ? 0 : (m.model == 1 ? 1 : 2);
        const int path = pair_of(m) ? ((m.g.nw & 1) ? 2 : 1) : 0;
        return fam * 9 + m.gm * 3 + path;
    };
    std::vector<int> order(nm);
    for (int i = 0; i < nm; ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) {
        const int sx = singles(M[x]), sy = singles(M[y]);
        return sx != sy ? sx > sy : code_of(M[x]) < code_of(M[y]);
    });
    std::vector<BatchEntry> E;
    std::vector<int> P(1, 0), nst;
    std::vector<size_t> key_off, member_key(nm, 0);
    size_t nkeys = 0;
    const int per_block = 8 * wt;
    for (int i : order) {
        Member &m = M[i];
        if (m.nsteps == 0) continue;
        BatchEntry e;
        std::memset(&e, 0, sizeof(e));
        e.a.solid = m.solid.data();
        e.a.slip = m.slip.data();
        e.a.chir = nullptr;
        e.a.g = m.g;
        e.a.chunks = (m.g.nw + 31) / 32;
        e.a.force_thr = m.fx >= 0 ? m.thr : 0;
        e.a.fx = m.fx;
        const bool pair = pair_of(m);
        e.a.wpt = pair ? 2 : 1;
        e.wpt = e.a.wpt;
        e.gm = m.gm;
        e.code = code_of(m);
        e.items = pair ? (m.g.nw + 1) / 2 : m.g.nw;
        e.a.fmagic = flat_magic(m.H, e.items);
        e.buf0 = m.buf[m.cur].data();
        e.buf1 = m.buf[m.cur ^ 1].data();
        e.seed = m.seed;
        e.t0 = m.t0;
        e.nsteps = m.nsteps;
        key_off.push_back(nkeys);
        member_key[i] = nkeys;
        nkeys += 2 * (size_t)m.nsteps;
        const long long own = singles(m) > 0 ? flat_tasks(m.H, e.items) : 0;
        e.task0 = P.back();
        e.tasks = (int)own;
        E.push_back(e);
        P.push_back((int)(P.back() + (own + per_block - 1) / per_block * per_block));
        nst.push_back(singles(m));
    }
    const int ne = (int)E.size();
    std::vector<uint64_t> keys(nkeys ? nkeys : 1);
    for (int l = 0; l < ne; ++l) E[l].keys = keys.data() + key_off[l];
    const int nblocks = ne ? P.back() / per_block : 0;
    std::vector<int> Bl(nblocks);
    for (int l = 0; l < ne; ++l)
        for (int b = P[l] / per_block; b < P[l + 1] / per_block; ++b) Bl[b] = l;
    int max_steps = 0, max_keys = 0;
    for (int l = 0; l < ne; ++l) max_steps = std::max(max_steps, nst[l]), max_keys = std::max(max_keys, E[l].nsteps);

    // keys of every (member, step): k_batch_keys on its grid
    {
        const long long work = (long long)ne * max_keys;
        const unsigned blocks = (unsigned)((work + 255) / 256);
        for (unsigned b = 0; b < blocks; ++b)
            for (unsigned t = 0; t < 256; ++t) {
                blockIdx = make_uint3(b, 0, 0);
                threadIdx = make_uint3(t, 0, 0);
                blockDim = dim3(256, 1, 1);
                k_batch_keys(E.data(), ne, max_keys);
            }
    }
    // segments of constant active sets, the step counter as in the graphs
    int s_base = 0;
    int s0 = 0;
    while (s0 < max_steps) {
        int k = 0;
        while (k < ne && nst[k] > s0) ++k;
        const int s1 = nst[k - 1], len = s1 - s0, tasks = P[k];
        int gmax = GEOM_NONE;
        for (int i = 0; i < k; ++i) gmax = std::max(gmax, E[i].gm);
        s_base = s0;
        for (int s = 0; s < len; ++s) {
            const unsigned blocks = (unsigned)(tasks / per_block);
            run_grid(blocks, [&] {
                auto launch = [&](auto tag) {
                    constexpr int T = decltype(tag)::value;
                    if (gmax == GEOM_NONE) k_batch<GEOM_NONE, T>(E.data(), Bl.data(), s, &s_base);
                    else if (gmax == GEOM_NOSLIP) k_batch<GEOM_NOSLIP, T>(E.data(), Bl.data(), s, &s_base);
                    else k_batch<GEOM_FULL, T>(E.data(), Bl.data(), s, &s_base);
                };
                switch (wt) {
                case 1: launch(std::integral_constant<int, 1>{}); break;
                case 2: launch(std::integral_constant<int, 2>{}); break;
                case 4: launch(std::integral_constant<int, 4>{}); break;
                default: launch(std::integral_constant<int, 8>{}); break;
                }
            });
        }
        s0 = s1;
    }
    // ---- the passes of the wavefront members, one list per depth
    for (const int K : {2, 4, 8}) {
        std::vector<int> wo;
        for (int i : order)
            if (M[i].K == K) wo.push_back(i);
        std::stable_sort(wo.begin(), wo.end(), [&](int x, int y) {
            const int px = M[x].nsteps / K, py = M[y].nsteps / K;
            return px != py ? px > py : code_of(M[x]) < code_of(M[y]);
        });
        std::vector<BatchEntry> WE;
        std::vector<int> WP(1, 0), wn;
        for (int i : wo) {
            Member &m = M[i];
            BatchEntry e;
            std::memset(&e, 0, sizeof(e));
            e.a.solid = m.solid.data();
            e.a.slip = m.slip.data();
            e.a.g = m.g;
            e.a.chunks = (m.g.nw + 31) / 32;
            e.a.force_thr = m.fx >= 0 ? m.thr : 0;
            e.a.fx = m.fx;
            e.gm = m.gm;
            e.code = code_of(m);
            e.buf0 = m.buf[m.cur].data();
            e.buf1 = m.buf[m.cur ^ 1].data();
            e.K = K;
            e.r = m.nsteps % K;
            e.S = 64;
            e.nstrips = (m.g.nw + 29) / 30;
            e.keys = keys.data() + member_key[i];
            const long long own = (long long)e.nstrips * ((m.H + e.S - 1) / e.S);
            e.task0 = WP.back();
            e.tasks = (int)own;
            WE.push_back(e);
            WP.push_back((int)(WP.back() + (own + 3) / 4 * 4));
            wn.push_back(m.nsteps / K);
        }
        const int we = (int)WE.size();
        std::vector<int> WB(we ? WP.back() / 4 : 0);
        for (int l = 0; l < we; ++l)
            for (int b = WP[l] / 4; b < WP[l + 1] / 4; ++b) WB[b] = l;
        const int passes = we ? wn[0] : 0;
        const int j_base = 0;
        for (int j = 0; j < passes; ++j) {
            int k = 0;
            while (k < we && wn[k] > j) ++k;
            int gmax = GEOM_NONE;
            for (int i = 0; i < k; ++i) gmax = std::max(gmax, WE[i].gm);
            run_grid((unsigned)(WP[k] / 4), [&] {
                auto launch = [&](auto tag) {
                    constexpr int KK = decltype(tag)::value;
                    if (gmax == GEOM_NONE) k_batch_wave<GEOM_NONE, KK>(WE.data(), WB.data(), j, &j_base);
                    else if (gmax == GEOM_NOSLIP) k_batch_wave<GEOM_NOSLIP, KK>(WE.data(), WB.data(), j, &j_base);
                    else k_batch_wave<GEOM_FULL, KK>(WE.data(), WB.data(), j, &j_base);
                };
                if (K == 2) launch(std::integral_constant<int, 2>{});
                else if (K == 4) launch(std::integral_constant<int, 4>{});
                else launch(std::integral_constant<int, 8>{});
            }, 128);
        }
    }
    for (auto &m : M) {
        const int swaps = m.K ? m.nsteps % m.K + m.nsteps / m.K : m.nsteps;
        if (swaps & 1) m.cur ^= 1;
    }

    f = std::fopen(argv[2], "wb");
    if (!f) return 2;
    for (auto &m : M) {
        const int D = num_dir(m.model);
        const std::vector<uint64_t> &res = m.buf[m.cur];
        for (int y = 0; y < m.H; ++y)
            for (int x = 0; x < m.W; ++x) {
                const size_t o = (size_t)y * m.g.pitch + (x >> 6);
                uint8_t c = 0;
                for (int d = 0; d < D; ++d)
                    c |= (uint8_t)(((res[d * m.g.ps + o] >> (x & 63)) & 1) << d);
                m.cells[(size_t)y * m.W + x] = c;
            }
        std::fwrite(m.cells.data(), 1, m.cells.size(), f);
    }
    std::fclose(f);
    return 0;
}
