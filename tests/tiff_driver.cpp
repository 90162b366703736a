// tiff_driver.cpp -- reads one 16-bit TIFF with the command line's reader
// (emida_gb300/cli/tiff.hpp, replacing src/load_tiff.hpp:14-53) and writes
// u32 width, u32 height, then the raster as u16 row-major; compiled by
// tests/test_tiff.py.
#include <cstdio>
#include <string>
#include <vector>

#include "../emida_gb300/cli/tiff.hpp"

int main(int argc, char **argv)
{
    if (argc != 3) return 2;
    std::string err;
    uint32_t w = 0, h = 0;
    if (!emida_cli::tiff_size(argv[1], w, h, err)) {
        std::fprintf(stderr, "%s\n", err.c_str());
        return 1;
    }
    std::vector<uint16_t> raster((size_t)w * h);
    if (!emida_cli::load_tiff(argv[1], raster.data(), w, h, err)) {
        std::fprintf(stderr, "%s\n", err.c_str());
        return 1;
    }
    FILE *out = std::fopen(argv[2], "wb");
    if (!out) return 2;
    std::fwrite(&w, sizeof w, 1, out);
    std::fwrite(&h, sizeof h, 1, out);
    std::fwrite(raster.data(), sizeof(uint16_t), raster.size(), out);
    std::fclose(out);
    return 0;
}
