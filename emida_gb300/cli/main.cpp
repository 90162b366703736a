// main.cpp -- the `emida` command line over libemida_gb.so.
//
// Flags, defaults, input files and output format follow the reference CLI
// (src/args_parser.cpp:113-283, src/args_parser.hpp:18-38,
// src/process_files.hpp:52-266, src/main.cpp:9-38):
//   -i,--initial TIFF   -d,--deformed LIST   -b,--slicepos ROIFILE
//   -s,--slicesize X,Y (radius)   -c,--crosssize X,Y   --precision double|float
//   -f,--fitsize 3|5|7|9   --crosspolicy brute|fft   --batchsize N   --loadworkers N
//   -q,--writecoefs   -a,--analysis   -o,--outpics DIR (accepted, unused as in the
//   reference)   --slicestep X,Y   --mode auto|plain|fused|tensor   -h,--help
// Output on stdout, per pattern: "%f %f %llu %s" (position, ROI count, file),
// then per ROI "%lu %lu %f %f" (mid, offset) or with -q six more "%f" coefficients.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstdio>
#include <fstream>
#include <future>
#include <iostream>
#include <limits>
#include <map>
#include <memory>
#include <mutex>
#include <queue>
#include <sstream>
#include <string>
#include <thread>
#include <vector>

#include "../../include/emida_gb/gpu_offset.hpp"
#include "text.hpp"
#include "tiff.hpp"

using namespace emida;

namespace {

struct params {
    std::string initial, deformed, slicepos, outdir;
    size2_t pic_size{0, 0}, cross_size{0, 0}, slice_size{64, 64};
    bool cross_given = false, slice_given = false;
    std::vector<size2_t> mids, begins;
    bool write_coefs = false, analysis = false, use_double = true;
    int fitsize = 3;
    cross_policy policy = CROSS_POLICY_FFT;
    esize_t batch = 1, workers = 1;
    int mode = EMIDA_GB_MODE_AUTO;
    std::string binary;  // results as binary records instead of text
};

const char *usage =
    "usage: emida -i TIFF_FILE -d TXT_FILE -b FILE_PATH [options]\n"
    "  -i,--initial TIFF_FILE     initial (reference) pattern\n"
    "  -d,--deformed TXT_FILE     list of deformed patterns, lines 'x y path'\n"
    "  -b,--slicepos FILE_PATH    ROI file: first line radius, then 'mid_x mid_y' lines\n"
    "  -s,--slicesize X,Y         ROI radius (overrides the ROI file)\n"
    "  -c,--crosssize X,Y         lag window (odd), brute policy only\n"
    "  -o,--outpics FOLDER        accepted, unused\n"
    "  --slicestep X,Y            cannot be combined with --slicepos\n"
    "  -a,--analysis              timings to standard error\n"
    "  -q,--writecoefs            also print the 6 fit coefficients\n"
    "  --precision double|float   (default double)\n"
    "  -f,--fitsize 3|5|7|9       (default 3)\n"
    "  --crosspolicy brute|fft    (default fft)\n"
    "  --batchsize N              patterns per batch (default 1)\n"
    "  --loadworkers N            pattern loading threads (default 1)\n"
    "  --mode auto|plain|fused|tensor  execution form (default auto; tensor: brute\n"
    "                             policy on the tensor cores, float, 64x64 ROIs)\n"
    "  --binary FILE              write the results to FILE as binary records (full\n"
    "                             precision) instead of text: per pattern f64 x, f64 y,\n"
    "                             u32 rois, u32 name bytes, name; per ROI u32 mid x,\n"
    "                             u32 mid y, f64 dx, f64 dy, f64 coefs[6] (little-endian)\n"
    "  -h,--help\n";

bool parse_pair(const std::string &v, size2_t &out)
{
    std::stringstream ss(v);
    std::string a, b;
    if (!std::getline(ss, a, ',') || !std::getline(ss, b, ',')) return false;
    try {
        out = {(esize_t)std::stoul(a), (esize_t)std::stoul(b)};
    } catch (...) {
        return false;
    }
    return true;
}

// src/args_parser.cpp:67-111
bool load_slice_mids(const std::string &file, size_t &radius, std::vector<size2_t> &mids)
{
    std::ifstream fin(file);
    if (!fin) {
        std::cerr << "Error: cannot open " << file << "\n";
        return false;
    }
    std::string line;
    std::getline(fin, line);
    try {
        radius = std::stoull(line);
    } catch (const std::exception &e) {
        std::cerr << "Warning: could not parse the first line with size of file " << file
                  << ". Error:'" << e.what() << "'. Skipping.\n";
    }
    int i = 0;
    while (std::getline(fin, line)) {
        ++i;
        const size_t split = line.find(' ');
        if (split == std::string::npos) {
            std::cerr << "Warning: could not parse line " << i << " of file " << file << ". Skipping.\n";
            continue;
        }
        try {
            mids.push_back({(esize_t)std::stoul(line.substr(0, split)),
                            (esize_t)std::stoul(line.substr(split + 1))});
        } catch (const std::exception &e) {
            std::cerr << "Warning: could not parse line " << i << " of file " << file << ". Error:'"
                      << e.what() << "'. Skipping.\n";
        }
    }
    return true;
}

bool parse(int argc, char **argv, params &a, bool &help)
{
    std::map<std::string, std::string> alias = {
        {"-i", "initial"}, {"-d", "deformed"}, {"-o", "outpics"}, {"-c", "crosssize"},
        {"-s", "slicesize"}, {"-b", "slicepos"}, {"-a", "analysis"}, {"-q", "writecoefs"},
        {"-f", "fitsize"}, {"-h", "help"}};
    const std::vector<std::string> flags = {"analysis", "writecoefs", "help"};
    std::map<std::string, std::string> v;
    for (int i = 1; i < argc; ++i) {
        std::string k = argv[i], val;
        if (alias.count(k)) k = alias[k];
        else if (k.rfind("--", 0) == 0) {
            k = k.substr(2);
            const size_t eq = k.find('=');
            if (eq != std::string::npos) {
                val = k.substr(eq + 1);
                k = k.substr(0, eq);
            }
        } else {
            std::cerr << "Argument parsing error.\n" << usage;
            return false;
        }
        const bool is_flag = std::find(flags.begin(), flags.end(), k) != flags.end();
        if (!is_flag && val.empty()) {
            if (i + 1 >= argc) {
                std::cerr << "Argument parsing error.\n" << usage;
                return false;
            }
            val = argv[++i];
        }
        v[k] = is_flag ? "1" : val;
    }
    if (v.count("help")) {
        help = true;
        std::cerr << usage;
        return true;
    }
    if (!v.count("initial") || !v.count("deformed") || !v.count("slicepos")) {
        std::cerr << "Argument parsing error.\n" << usage;
        return false;
    }
    a.initial = v["initial"];
    a.deformed = v["deformed"];
    if (v.count("outpics")) a.outdir = v["outpics"];
    if (v.count("slicesize")) {
        if (!parse_pair(v["slicesize"], a.slice_size)) return false;
        a.slice_size = a.slice_size * 2u;
        a.slice_given = true;
    }
    if (v.count("slicestep")) {
        std::cerr << "Error: cannot use slicestep when slicepos specified\n";
        return false;
    }
    size_t radius = 0;
    if (!load_slice_mids(v["slicepos"], radius, a.mids)) return false;
    if (a.slice_given)
        std::cerr << "Warning: size written in --slicepos file will be overriden by --slicesize.\n";
    else
        a.slice_size = {(esize_t)radius * 2u, (esize_t)radius * 2u};
    for (const auto &m : a.mids) {
        if (m.x < a.slice_size.x / 2 || m.y < a.slice_size.y / 2) {
            std::cerr << "Error: A slice out of bounds\n";
            return false;
        }
        a.begins.push_back({m.x - a.slice_size.x / 2, m.y - a.slice_size.y / 2});
    }
    if (v.count("crosssize")) {
        if (!parse_pair(v["crosssize"], a.cross_size)) return false;
        a.cross_given = true;
    } else {
        a.cross_size = {a.slice_size.x * 2 - 1, a.slice_size.y * 2 - 1};
    }
    if (a.cross_size.x > a.slice_size.x * 2 - 1 || a.cross_size.y > a.slice_size.y * 2 - 1) {
        std::cerr << "Error: cross size must be lesser or equal to slice_size * 2 - 1.\n";
        return false;
    }
    if (v.count("precision")) {
        if (v["precision"] == "float") a.use_double = false;
        else if (v["precision"] == "double") a.use_double = true;
        else {
            std::cerr << "Invalid precision argument.\n";
            return false;
        }
    }
    if (v.count("fitsize")) {
        a.fitsize = std::atoi(v["fitsize"].c_str());
        if (a.fitsize != 3 && a.fitsize != 5 && a.fitsize != 7 && a.fitsize != 9) {
            std::cerr << "Error: the fitsize " << a.fitsize << " is not supported.\n";
            return false;
        }
    }
    if (v.count("crosspolicy")) {
        if (v["crosspolicy"] == "fft") {
            a.policy = CROSS_POLICY_FFT;
            if (a.cross_given) std::cerr << "Warning: --crosssize (-c) is ignored with FFT policy.\n";
        } else if (v["crosspolicy"] == "brute")
            a.policy = CROSS_POLICY_BRUTE;
        else {
            std::cerr << "Invalid crosspolicy argument.\n";
            return false;
        }
    }
    // The reference returns success from parse() on a bad batchsize / loadworkers
    // (src/args_parser.cpp:257-258, 269-270); this CLI rejects them.
    if (v.count("batchsize")) {
        const int b = std::atoi(v["batchsize"].c_str());
        if (b <= 0) {
            std::cerr << "Error: batchsize must be greater than 0.\n";
            return false;
        }
        a.batch = (esize_t)b;
    }
    if (v.count("loadworkers")) {
        const int w = std::atoi(v["loadworkers"].c_str());
        if (w <= 0) {
            std::cerr << "Error: loadworkers must be greater than 0.\n";
            return false;
        }
        a.workers = (esize_t)w;
    }
    if (v.count("mode")) {
        const std::string m = v["mode"];
        a.mode = m == "plain" ? EMIDA_GB_MODE_PLAIN
                 : m == "fused" ? EMIDA_GB_MODE_FUSED
                 : m == "tensor" ? EMIDA_GB_MODE_TENSOR
                                 : EMIDA_GB_MODE_AUTO;
    }
    if (v.count("binary")) a.binary = v["binary"];
    a.analysis = v.count("analysis") > 0;
    a.write_coefs = v.count("writecoefs") > 0;
    std::string err;
    uint32_t w, h;
    if (!emida_cli::tiff_size(a.initial, w, h, err)) {
        std::cerr << err << "\n";
        return false;
    }
    a.pic_size = {w, h};
    return true;
}

// Label -> (sum ms, count), printed as "label: mean ms" (src/stopwatch.hpp:95-101).
struct timings {
    std::mutex mu;
    std::map<std::string, std::pair<double, long>> t;
    bool on = false;
    void add(const std::string &label, double ms)
    {
        if (!on) return;
        std::lock_guard<std::mutex> lk(mu);
        auto &e = t[label];
        e.first += ms;
        e.second += 1;
    }
    void write()
    {
        for (auto &e : t) std::cerr << e.first << ": " << e.second.first / e.second.second << "ms\n";
    }
} g_time;

struct stopwatch {
    std::chrono::steady_clock::time_point s = std::chrono::steady_clock::now();
    void tick(const std::string &label)
    {
        const auto n = std::chrono::steady_clock::now();
        g_time.add(label, std::chrono::duration<double, std::milli>(n - s).count());
        s = n;
    }
};

template <typename T>
struct bounded_queue {
    std::queue<T> q;
    std::mutex mu;
    std::condition_variable not_empty, not_full;
    size_t cap;
    explicit bounded_queue(size_t c) : cap(c) {}
    void push(T v)
    {
        std::unique_lock<std::mutex> lk(mu);
        not_full.wait(lk, [&] { return q.size() < cap; });
        q.push(std::move(v));
        not_empty.notify_one();
    }
    T pop()
    {
        std::unique_lock<std::mutex> lk(mu);
        not_empty.wait(lk, [&] { return !q.empty(); });
        T v = std::move(q.front());
        q.pop();
        not_full.notify_one();
        return v;
    }
};

struct work_item {
    double x, y;
    std::string fname;
};

// src/process_files.hpp:56-75
std::vector<work_item> load_work(const std::string &file)
{
    std::vector<work_item> r;
    std::ifstream in(file);
    std::string line;
    while (std::getline(in, line)) {
        work_item w;
        std::stringstream ss(line);
        ss >> w.x >> w.y;
        ss.ignore();
        std::getline(ss, w.fname);
        if (!ss.fail() || !w.fname.empty()) r.push_back(w);
    }
    return r;
}

template <typename T>
int process(const params &a)
{
    stopwatch sw;
    const size_t area = (size_t)a.pic_size.x * a.pic_size.y;
    std::vector<uint16_t> initial(area);
    std::string err;
    if (!emida_cli::load_tiff(a.initial, initial.data(), a.pic_size.x, a.pic_size.y, err)) {
        std::cerr << err << "\n";
        return 1;
    }
    const esize_t S = (esize_t)a.begins.size(), B = a.batch;
    gpu_offset<T, uint16_t> offs(a.pic_size, &a.begins, a.slice_size, a.cross_size, B, a.policy,
                                 a.fitsize, 2 * a.workers, a.mode);
    offs.allocate_memory(initial.data());
    const std::vector<work_item> work = load_work(a.deformed);
    if (work.empty()) {
        std::cerr << "The deformed list is empty.\n";
        return 0;
    }
    sw.tick("initialization");

    struct batch_job {
        esize_t first, files, buffer;
        bool ok;
    };
    struct fin_job {
        esize_t first, files;
        std::vector<data_index<T>> maxes;
        std::vector<T> neigh;
    };
    const esize_t n_batches = (esize_t)((work.size() + B - 1) / B);
    bounded_queue<batch_job> loaded(a.workers);
    bounded_queue<std::shared_ptr<fin_job>> done(2);
    std::atomic<esize_t> next{0};
    std::vector<uint16_t *> pinned(a.workers * 2 + 2, nullptr);
    for (auto &p : pinned) {
        void *h = nullptr;
        check_status(emida_gb_malloc_host(&h, area * B * sizeof(uint16_t)));
        p = (uint16_t *)h;
    }
    std::atomic<size_t> pin_next{0};
    std::mutex order_mu;
    std::condition_variable order_cv;
    esize_t next_to_submit = 0;

    // The rows that hold ROI pixels, merged into ascending bands: the path
    // copies and reads nothing else of a pattern, so the loaders read only
    // these (unless they cover nearly all of it).
    std::vector<std::pair<uint32_t, uint32_t>> bands;
    {
        std::vector<std::pair<uint32_t, uint32_t>> iv;
        for (const auto &b : a.begins)
            iv.push_back({(uint32_t)b.y, (uint32_t)std::min<size_t>(a.pic_size.y, b.y + a.slice_size.y)});
        std::sort(iv.begin(), iv.end());
        uint64_t covered = 0;
        for (const auto &r : iv) {
            if (!bands.empty() && r.first <= bands.back().first + bands.back().second) {
                const uint32_t end = std::max(bands.back().first + bands.back().second, r.second);
                bands.back().second = end - bands.back().first;
            } else if (r.second > r.first) {
                bands.push_back({r.first, r.second - r.first});
            }
        }
        for (const auto &bd : bands) covered += bd.second;
        if (covered * 10 >= (uint64_t)a.pic_size.y * 9) bands.clear();  // read whole patterns
    }
    // loaders (src/process_files.hpp:98-133): batches are submitted in order
    auto loader = [&]() {
        esize_t bi;
        while ((bi = next.fetch_add(1)) < n_batches) {
            stopwatch lsw;
            const esize_t first = bi * B;
            const esize_t files = std::min<esize_t>(B, (esize_t)work.size() - first);
            uint16_t *buf = pinned[pin_next.fetch_add(1) % pinned.size()];
            bool ok = true;
            for (esize_t i = 0; i < files; ++i) {
                std::string e;
                const bool got = bands.empty()
                                     ? emida_cli::load_tiff(work[first + i].fname, buf + i * area, a.pic_size.x,
                                                            a.pic_size.y, e)
                                     : emida_cli::load_tiff_rows(work[first + i].fname, buf + i * area,
                                                                 a.pic_size.x, a.pic_size.y, bands, e);
                if (!got) {
                    std::cerr << e << "\n";
                    ok = false;
                }
            }
            if (files < B) std::fill(buf + files * area, buf + B * area, (uint16_t)0);
            lsw.tick("Load tiff");
            std::unique_lock<std::mutex> lk(order_mu);
            order_cv.wait(lk, [&] { return next_to_submit == bi; });
            esize_t buffer = 0;
            if (ok) buffer = offs.transfer_pic_to_device_async(buf);
            lsw.tick("Pic to device async");
            loaded.push({first, files, buffer, ok});
            ++next_to_submit;
            order_cv.notify_all();
        }
    };
    // the binary results file is opened before any worker starts, so a failure
    // leaves no thread running
    FILE *bin = nullptr;
    if (!a.binary.empty() && !(bin = fopen(a.binary.c_str(), "wb"))) {
        std::cerr << "Error: cannot open " << a.binary << " for writing\n";
        return 1;
    }
    // GPU stage (src/process_files.hpp:184-216)
    std::thread gpu([&]() {
        for (esize_t b = 0; b < n_batches; ++b) {
            stopwatch gsw;
            batch_job j = loaded.pop();
            gsw.tick("Offset wait");
            auto f = std::make_shared<fin_job>();
            f->first = j.first;
            f->files = j.ok ? j.files : 0;
            if (j.ok) {
                f->maxes.resize((size_t)S * B);
                f->neigh.resize((size_t)S * B * a.fitsize * a.fitsize);
                offs.get_offset_core(f->maxes.data(), f->neigh.data(), j.buffer);
            }
            gsw.tick("Offset");
            done.push(f);
        }
    });
    // finalize stage (src/process_files.hpp:219-264)
    // One pattern's lines: "%f %f %llu %s\n", then per ROI "%lu %lu %f %f"
    // (+ 6 x " %f" with -q).
    auto pattern_text = [&](const offsets_t<double> &r, esize_t first, esize_t j, std::string &text) {
        using emida_cli::put_f;
        using emida_cli::put_u;
        put_f(text, work[j].x);
        text += ' ';
        put_f(text, work[j].y);
        text += ' ';
        put_u(text, (unsigned long long)S);
        text += ' ';
        text += work[j].fname;
        text += '\n';
        const esize_t it = j - first;
        for (esize_t i = it * S; i < (it + 1) * S; ++i) {
            const esize_t bi = i % S;
            double ox = r.offsets[i].x, oy = r.offsets[i].y;
            if (std::isnan(ox)) ox = std::numeric_limits<double>::quiet_NaN();
            if (std::isnan(oy)) oy = std::numeric_limits<double>::quiet_NaN();
            put_u(text, (unsigned long)a.mids[bi].x);
            text += ' ';
            put_u(text, (unsigned long)a.mids[bi].y);
            text += ' ';
            put_f(text, ox);
            text += ' ';
            put_f(text, oy);
            if (a.write_coefs)
                for (int k = 0; k < 6; ++k) {
                    text += ' ';
                    put_f(text, r.coefs[i][k]);
                }
            text += '\n';
        }
    };
    // a batch's text is formatted in up to TEXT_PARTS ranges of its patterns
    // at once (seven helper threads and this one), then written in order
    constexpr esize_t TEXT_PARTS = 8;
    std::thread fin([&]() {
        std::vector<std::string> parts(TEXT_PARTS);
        for (esize_t b = 0; b < n_batches; ++b) {
            stopwatch fsw;
            auto f = done.pop();
            fsw.tick("Finalize wait");
            if (f->files == 0) continue;  // a batch that failed to load is skipped
            auto r = offs.finalize(f->maxes.data(), f->neigh.data());
            if (bin) {
                for (esize_t j = f->first; j < f->first + f->files; ++j) {
                    // the same content, unrounded: pattern header, then one record per ROI
                    const uint32_t n = (uint32_t)S, len = (uint32_t)work[j].fname.size();
                    fwrite(&work[j].x, sizeof(double), 1, bin);
                    fwrite(&work[j].y, sizeof(double), 1, bin);
                    fwrite(&n, sizeof n, 1, bin);
                    fwrite(&len, sizeof len, 1, bin);
                    fwrite(work[j].fname.data(), 1, len, bin);
                    const esize_t it = j - f->first;
                    for (esize_t i = it * S; i < (it + 1) * S; ++i) {
                        const uint32_t mid[2] = {(uint32_t)a.mids[i % S].x, (uint32_t)a.mids[i % S].y};
                        const double o[2] = {r.offsets[i].x, r.offsets[i].y};
                        fwrite(mid, sizeof mid, 1, bin);
                        fwrite(o, sizeof o, 1, bin);
                        fwrite(r.coefs[i].data(), sizeof(double), 6, bin);
                    }
                }
                fsw.tick("Finalize");
                continue;
            }
            const esize_t nparts = std::min<esize_t>(TEXT_PARTS, f->files);
            auto format = [&](esize_t p) {
                const esize_t j0 = f->first + f->files * p / nparts;
                const esize_t j1 = f->first + f->files * (p + 1) / nparts;
                parts[p].clear();
                parts[p].reserve((size_t)(j1 - j0) * S * (a.write_coefs ? 120 : 40));
                for (esize_t j = j0; j < j1; ++j) pattern_text(r, f->first, j, parts[p]);
            };
            std::vector<std::future<void>> helpers;
            for (esize_t p = 1; p < nparts; ++p) helpers.push_back(std::async(std::launch::async, format, p));
            format(0);
            for (auto &h : helpers) h.get();
            for (esize_t p = 0; p < nparts; ++p)
                if (!parts[p].empty()) fwrite(parts[p].data(), 1, parts[p].size(), stdout);
            fsw.tick("Finalize");
        }
    });
    std::vector<std::thread> loaders;
    for (esize_t i = 1; i < a.workers; ++i) loaders.emplace_back(loader);
    loader();
    for (auto &t : loaders) t.join();
    gpu.join();
    fin.join();
    if (bin && fclose(bin) != 0) {
        std::cerr << "Error: writing " << a.binary << " failed\n";
        return 1;
    }
    for (auto p : pinned) emida_gb_free_host(p);
    fflush(stdout);
    return 0;
}

}  // namespace

int main(int argc, char **argv)
{
    params a;
    bool help = false;
    if (!parse(argc, argv, a, help)) return 1;
    if (help) return 0;
    g_time.on = a.analysis;
    int rc;
    try {
        rc = a.use_double ? process<double>(a) : process<float>(a);
    } catch (std::runtime_error &e) {
        std::cout << "Error: " << e.what() << "\n";
        return 1;
    }
    if (a.analysis) g_time.write();
    return rc;
}
