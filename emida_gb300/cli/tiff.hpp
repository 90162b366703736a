// tiff.hpp -- minimal reader/writer for uncompressed 16-bit grayscale TIFF
// strips, the only kind the reference loads (src/load_tiff.hpp:14-69, which
// copies raw strips through libtiff).  Both byte orders are read; big-endian
// pixels are swapped to host order.
#pragma once

#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

namespace emida_cli {

struct tiff_info {
    uint32_t width = 0, height = 0;
    uint16_t bits = 0, compression = 1, samples = 1, orientation = 1;
    bool big_endian = false;
    std::vector<uint64_t> strip_offsets, strip_bytes;
};

class tiff_file {
    FILE *f_ = nullptr;
    bool be_ = false;

    bool rd(uint64_t off, void *dst, size_t n)
    {
        return fseek(f_, (long)off, SEEK_SET) == 0 && fread(dst, 1, n, f_) == n;
    }
    uint16_t u16(const unsigned char *p) const
    {
        return be_ ? (uint16_t)((p[0] << 8) | p[1]) : (uint16_t)(p[0] | (p[1] << 8));
    }
    uint32_t u32(const unsigned char *p) const
    {
        return be_ ? ((uint32_t)p[0] << 24) | ((uint32_t)p[1] << 16) | ((uint32_t)p[2] << 8) | p[3]
                   : (uint32_t)p[0] | ((uint32_t)p[1] << 8) | ((uint32_t)p[2] << 16) |
                         ((uint32_t)p[3] << 24);
    }
    // values of a SHORT or LONG field (inline or at an offset)
    bool values(uint16_t type, uint32_t count, const unsigned char *inl, std::vector<uint64_t> &out)
    {
        const size_t sz = type == 3 ? 2 : 4;
        if (type != 3 && type != 4) return false;
        std::vector<unsigned char> buf(sz * count);
        if (sz * count <= 4)
            std::memcpy(buf.data(), inl, sz * count);
        else if (!rd(u32(inl), buf.data(), buf.size()))
            return false;
        out.resize(count);
        for (uint32_t i = 0; i < count; ++i)
            out[i] = sz == 2 ? u16(&buf[2 * i]) : u32(&buf[4 * i]);
        return true;
    }

public:
    ~tiff_file()
    {
        if (f_) fclose(f_);
    }

    bool open(const std::string &name, tiff_info &info, std::string &err)
    {
        f_ = fopen(name.c_str(), "rb");
        if (!f_) {
            err = "cannot open " + name;
            return false;
        }
        unsigned char h[8];
        if (!rd(0, h, 8) || !((h[0] == 'I' && h[1] == 'I') || (h[0] == 'M' && h[1] == 'M'))) {
            err = name + " is not a TIFF file";
            return false;
        }
        be_ = h[0] == 'M';
        info.big_endian = be_;
        if (u16(h + 2) != 42) {
            err = name + ": unsupported TIFF variant";
            return false;
        }
        const uint32_t ifd = u32(h + 4);
        unsigned char nb[2];
        if (!rd(ifd, nb, 2)) {
            err = name + ": truncated IFD";
            return false;
        }
        const uint16_t n = u16(nb);
        std::vector<unsigned char> ent(12 * (size_t)n);
        if (!rd(ifd + 2, ent.data(), ent.size())) {
            err = name + ": truncated IFD";
            return false;
        }
        for (uint16_t i = 0; i < n; ++i) {
            const unsigned char *e = &ent[12 * (size_t)i];
            const uint16_t tag = u16(e), type = u16(e + 2);
            const uint32_t count = u32(e + 4);
            std::vector<uint64_t> v;
            if (!values(type, count, e + 8, v)) continue;
            switch (tag) {
            case 256: info.width = (uint32_t)v[0]; break;
            case 257: info.height = (uint32_t)v[0]; break;
            case 258: info.bits = (uint16_t)v[0]; break;
            case 259: info.compression = (uint16_t)v[0]; break;
            case 273: info.strip_offsets = v; break;
            case 274: info.orientation = (uint16_t)v[0]; break;
            case 277: info.samples = (uint16_t)v[0]; break;
            case 279: info.strip_bytes = v; break;
            default: break;
            }
        }
        return true;
    }

    // Reads the pixels into raster (width*height uint16).
    bool read(const tiff_info &info, uint16_t *raster, std::string &err)
    {
        if (info.bits != 16 || info.samples != 1 || info.compression != 1) {
            err = "only uncompressed 16-bit single-channel TIFF is supported";
            return false;
        }
        if (info.orientation != 1) {
            err = "only able to process row 0 TOP, col 0 LEFT orientation";
            return false;
        }
        if (info.strip_offsets.size() != info.strip_bytes.size()) {
            err = "inconsistent strip tables";
            return false;
        }
        const uint64_t total = (uint64_t)info.width * info.height * 2;
        uint64_t at = 0;
        // strips that follow each other in the file are read with one call
        for (size_t s = 0; s < info.strip_offsets.size() && at < total;) {
            const uint64_t off = info.strip_offsets[s];
            uint64_t n = 0;
            size_t e = s;
            while (e < info.strip_offsets.size() && at + n < total && info.strip_offsets[e] == off + n)
                n += info.strip_bytes[e++];
            if (at + n > total) n = total - at;
            if (!rd(off, (unsigned char *)raster + at, (size_t)n)) {
                err = "truncated strip data";
                return false;
            }
            at += n;
            s = e;
        }
        if (at != total) {
            err = "strip data shorter than the image";
            return false;
        }
        if (be_)
            for (uint64_t i = 0; i < total / 2; ++i) raster[i] = (uint16_t)((raster[i] >> 8) | (raster[i] << 8));
        return true;
    }

    // Reads only the rows of `bands` ((first row, rows) pairs, ascending and
    // disjoint) into raster (width*height uint16), with one read per run of
    // strips that follow each other in the file; the other rows of raster are
    // left as they are.
    bool read_rows(const tiff_info &info, uint16_t *raster,
                   const std::vector<std::pair<uint32_t, uint32_t>> &bands, std::string &err)
    {
        if (info.bits != 16 || info.samples != 1 || info.compression != 1) {
            err = "only uncompressed 16-bit single-channel TIFF is supported";
            return false;
        }
        if (info.orientation != 1) {
            err = "only able to process row 0 TOP, col 0 LEFT orientation";
            return false;
        }
        const size_t ns = info.strip_offsets.size();
        if (ns != info.strip_bytes.size()) {
            err = "inconsistent strip tables";
            return false;
        }
        const uint64_t row = (uint64_t)info.width * 2, total = row * info.height;
        std::vector<uint64_t> start(ns + 1, 0);  // raster byte of each strip
        for (size_t s = 0; s < ns; ++s) start[s + 1] = start[s] + info.strip_bytes[s];
        if (start[ns] < total) {
            err = "strip data shorter than the image";
            return false;
        }
        size_t s = 0;
        for (const auto &bd : bands) {
            uint64_t lo = (uint64_t)bd.first * row;
            const uint64_t hi = std::min<uint64_t>(total, (uint64_t)(bd.first + bd.second) * row);
            while (lo < hi) {
                while (s < ns && start[s + 1] <= lo) ++s;  // the strip that holds byte lo
                if (s == ns) {
                    err = "truncated strip data";
                    return false;
                }
                size_t e = s;
                while (start[e + 1] < hi && e + 1 < ns &&
                       info.strip_offsets[e + 1] == info.strip_offsets[e] + info.strip_bytes[e])
                    ++e;
                const uint64_t end = std::min(hi, start[e + 1]);
                if (!rd(info.strip_offsets[s] + (lo - start[s]), (unsigned char *)raster + lo, (size_t)(end - lo))) {
                    err = "truncated strip data";
                    return false;
                }
                if (be_)
                    for (uint64_t i = lo / 2; i < end / 2; ++i)
                        raster[i] = (uint16_t)((raster[i] >> 8) | (raster[i] << 8));
                lo = end;
            }
        }
        return true;
    }
};

// src/load_tiff.hpp:55-69 get_size
inline bool tiff_size(const std::string &name, uint32_t &w, uint32_t &h, std::string &err)
{
    tiff_file t;
    tiff_info info;
    if (!t.open(name, info, err)) return false;
    w = info.width;
    h = info.height;
    return true;
}

// src/load_tiff.hpp:14-53 load_tiff
inline bool load_tiff(const std::string &name, uint16_t *raster, uint32_t w, uint32_t h,
                      std::string &err)
{
    tiff_file t;
    tiff_info info;
    if (!t.open(name, info, err)) return false;
    if (info.width != w || info.height != h) {
        err = "The size of " + name + " is different than specified size " + std::to_string(w) +
              "," + std::to_string(h);
        return false;
    }
    return t.read(info, raster, err);
}

// load_tiff for the rows of `bands` only (ascending, disjoint (first, rows)
// pairs): the rows that hold ROI pixels, which are all the path reads.
inline bool load_tiff_rows(const std::string &name, uint16_t *raster, uint32_t w, uint32_t h,
                           const std::vector<std::pair<uint32_t, uint32_t>> &bands, std::string &err)
{
    tiff_file t;
    tiff_info info;
    if (!t.open(name, info, err)) return false;
    if (info.width != w || info.height != h) {
        err = "The size of " + name + " is different than specified size " + std::to_string(w) +
              "," + std::to_string(h);
        return false;
    }
    return t.read_rows(info, raster, bands, err);
}

// Writes an uncompressed little-endian 16-bit grayscale TIFF with one strip.
inline bool write_tiff(const std::string &name, const uint16_t *raster, uint32_t w, uint32_t h)
{
    FILE *f = fopen(name.c_str(), "wb");
    if (!f) return false;
    const uint32_t n_ent = 9, ifd = 8, data = ifd + 2 + 12 * n_ent + 4;
    auto put16 = [&](uint16_t v) { fputc(v & 0xff, f), fputc(v >> 8, f); };
    auto put32 = [&](uint32_t v) { put16((uint16_t)(v & 0xffff)), put16((uint16_t)(v >> 16)); };
    auto entry = [&](uint16_t tag, uint16_t type, uint32_t count, uint32_t value) {
        put16(tag), put16(type), put32(count);
        if (type == 3 && count == 1)
            put16((uint16_t)value), put16(0);
        else
            put32(value);
    };
    fputc('I', f), fputc('I', f), put16(42), put32(ifd);
    put16((uint16_t)n_ent);
    entry(256, 4, 1, w);
    entry(257, 4, 1, h);
    entry(258, 3, 1, 16);
    entry(259, 3, 1, 1);
    entry(262, 3, 1, 1);
    entry(273, 4, 1, data);
    entry(277, 3, 1, 1);
    entry(278, 4, 1, h);
    entry(279, 4, 1, w * h * 2);
    put32(0);
    const bool ok = fwrite(raster, 2, (size_t)w * h, f) == (size_t)w * h;
    fclose(f);
    return ok;
}

}  // namespace emida_cli
