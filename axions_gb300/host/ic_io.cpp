// Field tables on the host: see ic_io.hpp.
#include "ic_io.hpp"

#include <algorithm>
#include <charconv>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <stdexcept>
#include <thread>

namespace axh {

namespace {

constexpr char MAGIC[8] = {'A', 'X', 'I', 'O', 'N', 'S', 'B', '1'};

struct File {
    FILE* f = nullptr;
    File(const std::string& path, const char* mode) : f(std::fopen(path.c_str(), mode)) {}
    ~File()
    {
        if (f) std::fclose(f);
    }
};

[[noreturn]] void fail(const std::string& msg) { throw std::runtime_error(msg); }

int threads_for(size_t work, size_t grain)
{
    const unsigned hc = std::max(1u, std::thread::hardware_concurrency());
    return (int)std::max<size_t>(1, std::min<size_t>(hc, work / grain));
}

std::vector<char> slurp(const std::string& path)
{
    File in(path, "rb");
    if (!in.f) fail("cannot read " + path);
    std::vector<char> buf;
    char tmp[1 << 16];
    size_t got;
    while ((got = std::fread(tmp, 1, sizeof tmp, in.f)) > 0) buf.insert(buf.end(), tmp, tmp + got);
    if (std::ferror(in.f)) fail("read error on " + path);
    return buf;
}

bool blank(char c) { return c == ' ' || c == '\t' || c == '\r'; }

// non-empty lines in [b, e)
int64_t count_rows(const char* b, const char* e)
{
    int64_t n = 0;
    bool content = false;
    for (const char* p = b; p < e; ++p) {
        if (*p == '\n') {
            n += content;
            content = false;
        } else if (!blank(*p)) {
            content = true;
        }
    }
    return n + content;
}

void read_text(const std::string& path, const std::vector<char>& buf, int cols, int64_t rows, std::vector<double>& dst)
{
    const char* base = buf.data();
    const size_t n = buf.size();
    const int T = threads_for(n, 1 << 20);
    std::vector<size_t> cut(T + 1, n);
    cut[0] = 0;
    for (int t = 1; t < T; ++t) {  // chunk starts at line beginnings
        size_t c = std::max(cut[t - 1], n * (size_t)t / (size_t)T);
        while (c < n && c > 0 && base[c - 1] != '\n') ++c;
        cut[t] = c;
    }
    std::vector<int64_t> first(T + 1, 0);
    {
        std::vector<std::thread> th;
        for (int t = 0; t < T; ++t)
            th.emplace_back([&, t] { first[t + 1] = count_rows(base + cut[t], base + cut[t + 1]); });
        for (auto& x : th) x.join();
    }
    for (int t = 0; t < T; ++t) first[t + 1] += first[t];
    if (first[T] != rows)
        fail(path + ": expected " + std::to_string(rows) + " lines of " + std::to_string(cols) + " values, found " +
             std::to_string(first[T]) + " lines");
    std::mutex mu;
    std::string err;
    auto parse = [&](int t) {
        const char* p = base + cut[t];
        const char* e = base + cut[t + 1];
        int64_t r = first[t];
        while (p < e) {
            const char* eol = (const char*)std::memchr(p, '\n', (size_t)(e - p));
            if (!eol) eol = e;
            int c = 0;
            bool any = false;
            while (p < eol) {
                while (p < eol && blank(*p)) ++p;
                if (p >= eol) break;
                any = true;
                if (*p == '+') ++p;
                double v = 0;
                const auto res = std::from_chars(p, eol, v);
                if (res.ec != std::errc() || (res.ptr < eol && !blank(*res.ptr)) || !std::isfinite(v) || c >= cols) {
                    std::lock_guard<std::mutex> lk(mu);
                    if (err.empty())
                        err = path + ": row " + std::to_string(r + 1) +
                              (c >= cols ? ": more than " + std::to_string(cols) + " values"
                                         : ": bad or non-finite value");
                    return;
                }
                dst[(size_t)c * (size_t)rows + (size_t)r] = v;
                ++c;
                p = res.ptr;
            }
            if (any) {
                if (c != cols) {
                    std::lock_guard<std::mutex> lk(mu);
                    if (err.empty())
                        err = path + ": row " + std::to_string(r + 1) + ": expected " + std::to_string(cols) +
                              " values, found " + std::to_string(c);
                    return;
                }
                ++r;
            }
            p = eol + 1;
        }
    };
    std::vector<std::thread> th;
    for (int t = 0; t < T; ++t) th.emplace_back(parse, t);
    for (auto& x : th) x.join();
    if (!err.empty()) fail(err);
}

void read_binary(const std::string& path, int cols, int64_t rows, std::vector<double>& dst)
{
    File in(path, "rb");
    if (!in.f) fail("cannot read " + path);
    char magic[8];
    int64_t hr = 0, hc = 0;
    if (std::fread(magic, 1, 8, in.f) != 8 || std::memcmp(magic, MAGIC, 8) != 0 ||
        std::fread(&hr, sizeof hr, 1, in.f) != 1 || std::fread(&hc, sizeof hc, 1, in.f) != 1)
        fail(path + ": not a binary field table");
    if (hr != rows || hc != cols)
        fail(path + ": table is " + std::to_string(hr) + " x " + std::to_string(hc) + ", expected " +
             std::to_string(rows) + " x " + std::to_string(cols));
    const int64_t block = std::max<int64_t>(1, (1 << 22) / cols);
    std::vector<double> row((size_t)block * cols);
    for (int64_t r0 = 0; r0 < rows; r0 += block) {
        const int64_t nr = std::min(block, rows - r0);
        if (std::fread(row.data(), sizeof(double), (size_t)(nr * cols), in.f) != (size_t)(nr * cols))
            fail(path + ": short binary table");
        for (int64_t r = 0; r < nr; ++r)
            for (int c = 0; c < cols; ++c) {
                const double v = row[(size_t)(r * cols + c)];
                if (!std::isfinite(v)) fail(path + ": row " + std::to_string(r0 + r + 1) + ": non-finite value");
                dst[(size_t)c * (size_t)rows + (size_t)(r0 + r)] = v;
            }
    }
    char extra;
    if (std::fread(&extra, 1, 1, in.f) == 1) fail(path + ": trailing data after the table");
}

}  // namespace

bool is_binary_table(const std::string& path)
{
    File in(path, "rb");
    char magic[8];
    return in.f && std::fread(magic, 1, 8, in.f) == 8 && std::memcmp(magic, MAGIC, 8) == 0;
}

void read_table(const std::string& path, int cols, int64_t rows, std::vector<double>& dst)
{
    dst.assign((size_t)cols * (size_t)rows, 0.0);
    if (is_binary_table(path)) read_binary(path, cols, rows, dst);
    else read_text(path, slurp(path), cols, rows, dst);
}

void write_table_text(const std::string& path, int cols, int64_t rows, const double* src, int digits)
{
    File out(path, "wb");
    if (!out.f) fail("cannot write " + path);
    const int64_t block = 1 << 20;
    const int T = threads_for((size_t)std::min(rows, block), 1 << 14);
    std::vector<std::string> part(T);
    for (int64_t r0 = 0; r0 < rows; r0 += block) {
        const int64_t nr = std::min(block, rows - r0);
        std::vector<std::thread> th;
        for (int t = 0; t < T; ++t)
            th.emplace_back([&, t] {
                const int64_t a = r0 + nr * t / T, b = r0 + nr * (t + 1) / T;
                std::string& s = part[t];
                s.clear();
                s.reserve((size_t)(b - a) * (size_t)cols * (size_t)(digits + 8));
                char num[64];
                for (int64_t r = a; r < b; ++r) {
                    for (int c = 0; c < cols; ++c) {
                        const double v = src[(size_t)c * (size_t)rows + (size_t)r];
                        const auto res = std::to_chars(num, num + sizeof num, v, std::chars_format::general, digits);
                        if (c) s.push_back(' ');
                        s.append(num, res.ptr);
                    }
                    s.push_back('\n');
                }
            });
        for (auto& x : th) x.join();
        for (int t = 0; t < T; ++t)
            if (std::fwrite(part[t].data(), 1, part[t].size(), out.f) != part[t].size()) fail("write error on " + path);
    }
}

void write_table_bin(const std::string& path, int cols, int64_t rows, const double* src)
{
    File out(path, "wb");
    if (!out.f) fail("cannot write " + path);
    const int64_t hc = cols;
    if (std::fwrite(MAGIC, 1, 8, out.f) != 8 || std::fwrite(&rows, sizeof rows, 1, out.f) != 1 ||
        std::fwrite(&hc, sizeof hc, 1, out.f) != 1)
        fail("write error on " + path);
    const int64_t block = std::max<int64_t>(1, (1 << 22) / cols);
    std::vector<double> row((size_t)block * cols);
    for (int64_t r0 = 0; r0 < rows; r0 += block) {
        const int64_t nr = std::min(block, rows - r0);
        for (int64_t r = 0; r < nr; ++r)
            for (int c = 0; c < cols; ++c) row[(size_t)(r * cols + c)] = src[(size_t)c * (size_t)rows + (size_t)(r0 + r)];
        if (std::fwrite(row.data(), sizeof(double), (size_t)(nr * cols), out.f) != (size_t)(nr * cols))
            fail("write error on " + path);
    }
}

}  // namespace axh
