// tiff_driver.cpp -- reads one 16-bit TIFF with the command line's reader
// (emida_gb300/cli/tiff.hpp, replacing src/load_tiff.hpp:14-53) and writes
// u32 width, u32 height, then the raster as u16 row-major; compiled by
// tests/test_tiff.py.  With further arguments "first:rows ..." it reads only
// those row bands (load_tiff_rows) into a raster that starts as 0xffff.
#include <cstdio>
#include <cstdlib>
#include <string>
#include <utility>
#include <vector>

#include "../emida_gb300/cli/tiff.hpp"

int main(int argc, char **argv)
{
    if (argc < 3) return 2;
    std::string err;
    uint32_t w = 0, h = 0;
    if (!emida_cli::tiff_size(argv[1], w, h, err)) {
        std::fprintf(stderr, "%s\n", err.c_str());
        return 1;
    }
    std::vector<uint16_t> raster((size_t)w * h, 0xffff);
    std::vector<std::pair<uint32_t, uint32_t>> bands;
    for (int i = 3; i < argc; ++i) {
        char *colon = nullptr;
        const unsigned long first = std::strtoul(argv[i], &colon, 10);
        if (!colon || *colon != ':') return 2;
        bands.push_back({(uint32_t)first, (uint32_t)std::strtoul(colon + 1, nullptr, 10)});
    }
    const bool ok = bands.empty() ? emida_cli::load_tiff(argv[1], raster.data(), w, h, err)
                                  : emida_cli::load_tiff_rows(argv[1], raster.data(), w, h, bands, err);
    if (!ok) {
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
