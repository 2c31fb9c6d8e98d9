/*
 * io.h -- headless output of lattice fields: VTK XML image files (.vti) with
 * the arrays of the reference's IoVti (keva92/lgca src/lgca_io_vti.cpp:37-144)
 * and colour-mapped PNG images of a field.  Self-contained C++ (no VTK, no
 * libpng, no zlib): the .vti arrays are stored as raw appended binary, the
 * PNG image data in stored (uncompressed) deflate blocks.
 *
 * VtiWriter::write(step, dir) writes, like IoVti::write:
 *   <dir>cell_res_<step>.vti  image of (dim_x+1) x (dim_y+1) points with cell
 *                             arrays "Cell density" (1) and "Cell momentum" (2)
 *   <dir>mean_res_<step>.vti  image of coarse_dim_x x coarse_dim_y points with
 *                             point arrays "Mean density" (1), "Mean momentum" (2)
 */
#ifndef LGCA_IO_H_
#define LGCA_IO_H_

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

namespace lgca_gb300 {

struct VtiArray {
    std::string name;
    int components;
    const float *data;
    size_t tuples;
};

// One VTK XML ImageData file; `cell_data` selects CellData (else PointData).
inline bool write_vti(const std::string &path, int nx, int ny, bool cell_data,
                      const std::vector<VtiArray> &arrays, const std::string &active)
{
    FILE *f = std::fopen(path.c_str(), "wb");
    if (!f) return false;
    const int ex = cell_data ? nx : nx - 1, ey = cell_data ? ny : ny - 1;
    std::fprintf(f, "<?xml version=\"1.0\"?>\n");
    std::fprintf(f, "<VTKFile type=\"ImageData\" version=\"1.0\" byte_order=\"LittleEndian\" "
                    "header_type=\"UInt64\">\n");
    std::fprintf(f, "  <ImageData WholeExtent=\"0 %d 0 %d 0 0\" Origin=\"0 0 0\" Spacing=\"1 1 1\">\n",
                 ex, ey);
    std::fprintf(f, "    <Piece Extent=\"0 %d 0 %d 0 0\">\n", ex, ey);
    const char *tag = cell_data ? "CellData" : "PointData";
    std::fprintf(f, "      <%s Scalars=\"%s\">\n", tag, active.c_str());
    uint64_t offset = 0;
    for (const VtiArray &a : arrays) {
        std::fprintf(f, "        <DataArray type=\"Float32\" Name=\"%s\" NumberOfComponents=\"%d\" "
                        "format=\"appended\" offset=\"%llu\"/>\n",
                     a.name.c_str(), a.components, (unsigned long long)offset);
        offset += 8 + a.tuples * a.components * sizeof(float);
    }
    std::fprintf(f, "      </%s>\n    </Piece>\n  </ImageData>\n", tag);
    std::fprintf(f, "  <AppendedData encoding=\"raw\">\n   _");
    for (const VtiArray &a : arrays) {
        const uint64_t nbytes = a.tuples * a.components * sizeof(float);
        std::fwrite(&nbytes, sizeof(nbytes), 1, f);
        std::fwrite(a.data, 1, nbytes, f);
    }
    std::fprintf(f, "\n  </AppendedData>\n</VTKFile>\n");
    return std::fclose(f) == 0;
}

// IoVti of the reference, headless: borrows the lattice's post-processed
// arrays (cell_density(), cell_momentum(), mean_density(), mean_momentum()).
template <class LatticeT>
class VtiWriter {
public:
    VtiWriter(LatticeT *lattice, const std::string scalars) : m_lattice(lattice), m_scalars(scalars) {}
    void set_scalars(const std::string scalars) { m_scalars = scalars; }
    void update() {}
    bool write(size_t step, const std::string dir = "./")
    {
        LatticeT &L = *m_lattice;
        const std::string cell = dir + "cell_res_" + std::to_string(step) + ".vti";
        const std::string mean = dir + "mean_res_" + std::to_string(step) + ".vti";
        const bool cell_active = m_scalars.rfind("Cell", 0) == 0;
        bool ok = write_vti(cell, L.dim_x(), L.dim_y(), true,
                            {{"Cell density", 1, L.cell_density(), L.num_cells()},
                             {"Cell momentum", 2, L.cell_momentum(), L.num_cells()}},
                            cell_active ? m_scalars : "Cell density");
        ok = write_vti(mean, L.coarse_dim_x(), L.coarse_dim_y(), false,
                       {{"Mean density", 1, L.mean_density(), L.num_coarse_cells()},
                        {"Mean momentum", 2, L.mean_momentum(), L.num_coarse_cells()}},
                       cell_active ? "Mean density" : m_scalars) && ok;
        return ok;
    }

private:
    LatticeT *m_lattice;
    std::string m_scalars;
};

// ---------------------------------------------------------------- PNG
namespace png_detail {

inline uint32_t crc32(const uint8_t *p, size_t n, uint32_t c = 0)
{
    // CRC-32 (ISO 3309 / PNG), bitwise; tables are not worth it for a few images
    c = ~c;
    for (size_t i = 0; i < n; ++i) {
        c ^= p[i];
        for (int k = 0; k < 8; ++k) c = (c >> 1) ^ (0xEDB88320u & (0u - (c & 1u)));
    }
    return ~c;
}

inline void put32(std::vector<uint8_t> &v, uint32_t x)
{
    v.push_back((uint8_t)(x >> 24));
    v.push_back((uint8_t)(x >> 16));
    v.push_back((uint8_t)(x >> 8));
    v.push_back((uint8_t)x);
}

inline void chunk(FILE *f, const char *type, const std::vector<uint8_t> &data)
{
    std::vector<uint8_t> buf;
    put32(buf, (uint32_t)data.size());
    buf.insert(buf.end(), type, type + 4);
    buf.insert(buf.end(), data.begin(), data.end());
    const uint32_t c = crc32(buf.data() + 4, buf.size() - 4);
    put32(buf, c);
    std::fwrite(buf.data(), 1, buf.size(), f);
}

}  // namespace png_detail

// RGB8 image, rows top to bottom, as a PNG: zlib stream of stored deflate
// blocks (RFC 1950/1951) with an Adler-32 trailer.
inline bool write_png_rgb(const std::string &path, int w, int h, const std::vector<uint8_t> &rgb)
{
    using namespace png_detail;
    FILE *f = std::fopen(path.c_str(), "wb");
    if (!f) return false;
    static const uint8_t sig[8] = {137, 80, 78, 71, 13, 10, 26, 10};
    std::fwrite(sig, 1, 8, f);
    std::vector<uint8_t> ihdr;
    put32(ihdr, (uint32_t)w);
    put32(ihdr, (uint32_t)h);
    ihdr.push_back(8);  // bit depth
    ihdr.push_back(2);  // colour type RGB
    ihdr.push_back(0);
    ihdr.push_back(0);
    ihdr.push_back(0);
    chunk(f, "IHDR", ihdr);
    // raw scanlines with filter byte 0
    std::vector<uint8_t> raw;
    raw.reserve((size_t)h * (3 * (size_t)w + 1));
    for (int y = 0; y < h; ++y) {
        raw.push_back(0);
        raw.insert(raw.end(), rgb.begin() + (size_t)y * 3 * w, rgb.begin() + (size_t)(y + 1) * 3 * w);
    }
    std::vector<uint8_t> z;
    z.push_back(0x78);
    z.push_back(0x01);
    uint32_t a = 1, b = 0;
    for (size_t pos = 0; pos < raw.size() || pos == 0;) {
        const size_t n = std::min<size_t>(65535, raw.size() - pos);
        const bool last = pos + n >= raw.size();
        z.push_back(last ? 1 : 0);
        z.push_back((uint8_t)(n & 0xff));
        z.push_back((uint8_t)(n >> 8));
        z.push_back((uint8_t)(~n & 0xff));
        z.push_back((uint8_t)((~n >> 8) & 0xff));
        for (size_t i = 0; i < n; ++i) {
            const uint8_t c = raw[pos + i];
            z.push_back(c);
            a = (a + c) % 65521u;
            b = (b + a) % 65521u;
        }
        pos += n;
        if (last) break;
    }
    put32(z, (b << 16) | a);
    chunk(f, "IDAT", z);
    chunk(f, "IEND", {});
    return std::fclose(f) == 0;
}

// Field (row 0 = bottom, as the lattice's y axis) colour-mapped between lo and
// hi with a blue-white-red ramp; rows are flipped so that +y points up.
inline bool write_png_field(const std::string &path, int w, int h, const float *field, float lo,
                            float hi)
{
    std::vector<uint8_t> rgb((size_t)w * h * 3);
    const float span = hi > lo ? hi - lo : 1.0f;
    for (int y = 0; y < h; ++y) {
        for (int x = 0; x < w; ++x) {
            float t = (field[(size_t)y * w + x] - lo) / span;
            t = t < 0 ? 0 : (t > 1 ? 1 : t);
            const float r = t < 0.5f ? 2 * t : 1.0f, g = t < 0.5f ? 2 * t : 2 * (1 - t),
                        bl = t < 0.5f ? 1.0f : 2 * (1 - t);
            uint8_t *px = &rgb[((size_t)(h - 1 - y) * w + x) * 3];
            px[0] = (uint8_t)std::lround(255 * r);
            px[1] = (uint8_t)std::lround(255 * g);
            px[2] = (uint8_t)std::lround(255 * bl);
        }
    }
    return write_png_rgb(path, w, h, rgb);
}

}  // namespace lgca_gb300

#endif /* LGCA_IO_H_ */
