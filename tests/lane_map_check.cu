// Host check of the lane mapping of the one-step and batch kernels
// (flat_tasks / flat_magic / flat_site in lgca_gb300/csrc/internal.cuh),
// built with nvcc and run on the CPU by tests/test_lane_map.py:
//   * the multiply-high in flat_magic equals the divide on every lane number
//     the mapping produces;
//   * the warp tasks of a lattice cover every (row, lane item) exactly once,
//     lanes past a parity class's end get a row >= H;
//   * the rows of a warp share one parity;
//   * consecutive lanes of one row hold consecutive items, and rows follow
//     each other in order, so the source lanes the step bodies shuffle from
//     -- the neighbouring item, or across the periodic seam the row's last /
//     first item -- hold exactly that item whenever they lie in the warp.
// Prints "OK" and exits 0, or prints the first failures and exits 1.
#include "../lgca_gb300/csrc/internal.cuh"

#include <cstdio>
#include <vector>

using namespace lgca_gpu;

static long long fails = 0;

#define CHECK(cond, ...)                                           \
    do {                                                           \
        if (!(cond)) {                                             \
            if (fails++ < 20) {                                    \
                std::printf("FAIL line %d: ", __LINE__);           \
                std::printf(__VA_ARGS__);                          \
                std::printf("\n");                                 \
            }                                                      \
        }                                                          \
    } while (0)

static void check_magic(int H, int items)
{
    const uint32_t m = flat_magic(H, items);
    const unsigned long long lmax = (unsigned long long)((H + 1) / 2) * (unsigned)items + 32u;
    if (items < 2 || lmax * (unsigned long long)items >= (1ull << 32)) {
        CHECK(m == 0u, "H=%d items=%d: magic %u where a divide is needed", H, items, m);
        return;
    }
    CHECK(m != 0u, "H=%d items=%d: no magic", H, items);
    for (unsigned long long l = 0; l <= lmax; ++l) {
        const unsigned r = (unsigned)((l * m) >> 32);
        if (r != l / (unsigned)items) {
            CHECK(false, "H=%d items=%d l=%llu: %u != %llu", H, items, l, r, l / items);
            return;
        }
    }
}

static void check_map(int H, int items)
{
    const uint32_t m = flat_magic(H, items);
    const long long tasks = flat_tasks(H, items);
    std::vector<int> seen((size_t)H * items, 0);
    int last_y = -1, last_t = -1, last_p = -1;
    for (long long k = 0; k < tasks; ++k) {
        int y[32], t[32];
        for (int lane = 0; lane < 32; ++lane) flat_site(k, lane, H, items, m, y[lane], t[lane]);
        int par = -1;
        bool padding = false;
        for (int lane = 0; lane < 32; ++lane) {
            CHECK(t[lane] >= 0 && t[lane] < items, "H=%d items=%d task %lld lane %d: item %d", H,
                  items, k, lane, t[lane]);
            if (y[lane] >= H) {  // past the end of a parity class
                padding = true;
                continue;
            }
            CHECK(!padding, "H=%d items=%d task %lld lane %d: a row after padding", H, items, k,
                  lane);
            CHECK(y[lane] >= 0, "H=%d items=%d: row %d", H, items, y[lane]);
            if (par < 0) par = y[lane] & 1;
            CHECK((y[lane] & 1) == par, "H=%d items=%d task %lld: mixed parity", H, items, k);
            ++seen[(size_t)y[lane] * items + t[lane]];
            // the lane numbering continues the previous lane's, within a class
            if (last_p == (y[lane] & 1)) {
                const bool next_item = y[lane] == last_y && t[lane] == last_t + 1;
                const bool next_row = y[lane] == last_y + 2 && t[lane] == 0 && last_t == items - 1;
                CHECK(next_item || next_row, "H=%d items=%d task %lld lane %d: (%d,%d) after (%d,%d)",
                      H, items, k, lane, y[lane], t[lane], last_y, last_t);
            } else {
                CHECK(t[lane] == 0 && y[lane] == (y[lane] & 1), "H=%d items=%d: class starts at (%d,%d)",
                      H, items, y[lane], t[lane]);
            }
            last_y = y[lane];
            last_t = t[lane];
            last_p = y[lane] & 1;
            // source lanes of the west / east words (seam: the row's last / first item)
            const int srcw = lane + (t[lane] == 0 ? items - 1 : -1);
            const int srce = lane + (t[lane] == items - 1 ? 1 - items : 1);
            const int wantw = t[lane] == 0 ? items - 1 : t[lane] - 1;
            const int wante = t[lane] == items - 1 ? 0 : t[lane] + 1;
            if (srcw >= 0 && srcw < 32)
                CHECK(y[srcw] == y[lane] && t[srcw] == wantw,
                      "H=%d items=%d task %lld lane %d: west source lane %d holds (%d,%d)", H, items,
                      k, lane, srcw, y[srcw], t[srcw]);
            if (srce >= 0 && srce < 32)
                CHECK(y[srce] == y[lane] && t[srce] == wante,
                      "H=%d items=%d task %lld lane %d: east source lane %d holds (%d,%d)", H, items,
                      k, lane, srce, y[srce], t[srce]);
        }
    }
    for (int yy = 0; yy < H; ++yy)
        for (int tt = 0; tt < items; ++tt)
            CHECK(seen[(size_t)yy * items + tt] == 1, "H=%d items=%d: (%d,%d) covered %d times", H,
                  items, yy, tt, seen[(size_t)yy * items + tt]);
}

int main()
{
    const int Hs[] = {1, 2, 3, 4, 5, 7, 8, 30, 31, 32, 33, 63, 64, 65, 100, 255, 256, 1023, 1024, 2047};
    for (int items = 1; items <= 70; ++items)
        for (int H : Hs) {
            check_magic(H, items);
            check_map(H, items);
        }
    // tall lattices of the batched and served workloads, and the magic's limits
    const int big[][2] = {{16384, 2}, {16384, 64}, {4096, 33}, {65536, 32}, {1 << 20, 64},
                          {1 << 22, 64}, {1 << 23, 2}};
    for (const auto &c : big) {
        check_magic(c[0], c[1]);
        if ((long long)c[0] * c[1] <= (1 << 22)) check_map(c[0], c[1]);
    }
    if (fails) {
        std::printf("%lld failures\n", fails);
        return 1;
    }
    std::printf("OK\n");
    return 0;
}
