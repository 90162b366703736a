// text.hpp -- the result lines of src/process_files.hpp:244-260 without
// printf: numbers go through std::to_chars, which C++17 specifies to give the
// characters printf gives in the "C" locale for the same conversion ("%f" is
// fixed notation with 6 decimals, "%lu"/"%llu" plain decimal), appended to
// one buffer per batch that is written with a single fwrite.
#pragma once

#include <charconv>
#include <cmath>
#include <cstdint>
#include <string>

namespace emida_cli {

// printf("%f", v)
inline void put_f(std::string &out, double v)
{
    if (std::isnan(v)) {
        out += std::signbit(v) ? "-nan" : "nan";
        return;
    }
    if (std::isinf(v)) {
        out += std::signbit(v) ? "-inf" : "inf";
        return;
    }
    char buf[400];  // the longest "%f" of a finite double is 316 characters
    const auto r = std::to_chars(buf, buf + sizeof buf, v, std::chars_format::fixed, 6);
    out.append(buf, r.ptr);
}

// printf("%lu", v) / printf("%llu", v)
inline void put_u(std::string &out, unsigned long long v)
{
    char buf[24];
    const auto r = std::to_chars(buf, buf + sizeof buf, v);
    out.append(buf, r.ptr);
}

}  // namespace emida_cli
