// Writes a small .vti pair and a PNG with the headless writers of
// include/lgca/io.h from known arrays; tests/test_apps.py parses them.
#include "lgca/io.h"
#include <cstdio>
#include <vector>
using namespace lgca_gb300;

struct FakeLattice {
    unsigned dim_x() const { return 5; }
    unsigned dim_y() const { return 3; }
    unsigned coarse_dim_x() const { return 2; }
    unsigned coarse_dim_y() const { return 1; }
    size_t num_cells() const { return 15; }
    size_t num_coarse_cells() const { return 2; }
    float cd[15], cm[30], md[2], mm[4];
    float *cell_density() { return cd; }
    float *cell_momentum() { return cm; }
    float *mean_density() { return md; }
    float *mean_momentum() { return mm; }
};

int main(int argc, char **argv)
{
    const std::string dir = argc > 1 ? argv[1] : "./";
    FakeLattice L;
    for (int i = 0; i < 15; ++i) L.cd[i] = (float)i;
    for (int i = 0; i < 30; ++i) L.cm[i] = 0.5f * i - 3.0f;
    L.md[0] = 1.25f; L.md[1] = 2.5f;
    for (int i = 0; i < 4; ++i) L.mm[i] = -0.75f * i;
    VtiWriter<FakeLattice> io(&L, "Cell density");
    if (!io.write(7, dir)) return 1;
    std::vector<float> f(70000);
    for (size_t i = 0; i < f.size(); ++i) f[i] = (float)(i % 97);
    if (!write_png_field(dir + "field.png", 350, 200, f.data(), 0.0f, 96.0f)) return 1;
    return 0;
}
