// asc-convert: builds the engine's graph files from an edge list, the job of
// the reference's converter (converter/converter.cpp:22-420) as one command.
//
//   asc-convert INPUT [--to LIST] [--out STEM] [--symmetrize] [--transpose]
//               [--weights ref|uniform[:LO:HI]|column] [--seed N] [--compat]
//
// INPUT is a text edge list ("src dst" or "src dst weight" per line; blank
// lines and lines starting with '#' or '%' are skipped) or, when it ends in
// ".toB", the reference's binary pair file (u32 src, u32 dst per edge).
// LIST is a comma list of toB, bcsr, bwcsr, bcsc, bcsr32 (default
// bcsr,bwcsr,bcsc); each output is STEM.<format>, STEM being INPUT without
// its extension, as the reference names its outputs.
//
// What matches the reference converter:
//   * V = largest id + 1 over sources and destinations (converter.cpp:102-125);
//   * E = number of edges, self-loops and duplicates kept;
//   * each list keeps the edges in input order (a stable counting sort, as the
//     reference's two passes over the pair file, converter.cpp:143-164);
//   * bcsc holds, per vertex, its in-edges' sources in input order plus the
//     out-degree block (converter.cpp:188-300);
//   * --weights ref draws rand() % 20 after srand(0), one value per edge in
//     input order, as convertByteToBWCSR does (converter.cpp:303-306, :396);
//   * --compat also reproduces the offset step "if (tempPointer == totalSize)
//     tempPointer--" (converter.cpp:131-138): every vertex after the last one
//     with edges then starts at E - 1, so a reader that derives degrees from
//     the offsets moves the last edge to vertex V - 1. Without --compat the
//     offsets are exact.
// What differs, on purpose: comment and blank lines are skipped (the
// reference's stringstream parse turns them into bogus edges), ids and line
// syntax are checked (exit status 2 with the line number), V is written as a
// full u64 in every layout, and the weighted pass reads only the edges that
// exist (the reference's second pass reads partSize entries regardless).
#include <errno.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <string>
#include <vector>

#include "ascetic.h"

namespace {

struct EdgeList {
    std::vector<uint32_t> src, dst, w;
    bool has_column = false;
};

[[noreturn]] void die(const char *fmt, const char *a = "", unsigned long long n = 0) {
    fprintf(stderr, "asc-convert: ");
    fprintf(stderr, fmt, a, n);
    fprintf(stderr, "\n");
    exit(2);
}

bool ends_with(const std::string &s, const char *suf) {
    const size_t n = strlen(suf);
    return s.size() >= n && s.compare(s.size() - n, n, suf) == 0;
}

// Parses one unsigned decimal field; false at end of line.
bool field(const char *&p, const char *end, unsigned long long &out, bool &bad) {
    while (p < end && (*p == ' ' || *p == '\t' || *p == ',' || *p == '\r')) p++;
    if (p >= end) return false;
    if (*p < '0' || *p > '9') {
        bad = true;
        return false;
    }
    unsigned long long v = 0;
    while (p < end && *p >= '0' && *p <= '9') {
        v = v * 10 + (unsigned long long)(*p - '0');
        if (v > 0xffffffffull) {
            bad = true;
            return false;
        }
        p++;
    }
    out = v;
    return true;
}

void read_text(const std::string &path, EdgeList &el) {
    FILE *f = fopen(path.c_str(), "rb");
    if (!f) die("%s: cannot open", path.c_str());
    std::vector<char> buf;
    {
        char chunk[1 << 16];
        size_t n;
        while ((n = fread(chunk, 1, sizeof(chunk), f)) > 0) buf.insert(buf.end(), chunk, chunk + n);
        fclose(f);
    }
    const char *p = buf.data(), *end = p + buf.size();
    unsigned long long line = 0;
    int columns = -1;
    while (p < end) {
        const char *eol = (const char *)memchr(p, '\n', (size_t)(end - p));
        if (!eol) eol = end;
        line++;
        const char *q = p;
        while (q < eol && (*q == ' ' || *q == '\t' || *q == '\r')) q++;
        if (q < eol && *q != '#' && *q != '%') {
            unsigned long long v[3];
            int n = 0;
            bool bad = false;
            while (n < 3 && field(q, eol, v[n], bad)) n++;
            unsigned long long extra;
            if (!bad && n == 3 && field(q, eol, extra, bad)) bad = true;
            if (bad || n < 2) die("%s: line %llu is not \"src dst [weight]\" with ids below 2^32", path.c_str(), line);
            if (v[0] == 0xffffffffull || v[1] == 0xffffffffull)
                die("%s: line %llu: vertex id 4294967295 leaves no room for V", path.c_str(), line);
            if (columns < 0) columns = n;
            else if (columns != n) die("%s: line %llu has a different number of columns", path.c_str(), line);
            el.src.push_back((uint32_t)v[0]);
            el.dst.push_back((uint32_t)v[1]);
            if (n == 3) el.w.push_back((uint32_t)v[2]);
        }
        p = eol + 1;
    }
    el.has_column = columns == 3;
}

void read_pairs(const std::string &path, EdgeList &el) {
    FILE *f = fopen(path.c_str(), "rb");
    if (!f) die("%s: cannot open", path.c_str());
    fseek(f, 0, SEEK_END);
    const long long size = ftell(f);
    fseek(f, 0, SEEK_SET);
    if (size < 0 || size % 8) die("%s: size is not a whole number of (u32 src, u32 dst) pairs", path.c_str());
    const size_t n = (size_t)size / 8;
    std::vector<uint32_t> raw(2 * n);
    if (n && fread(raw.data(), 8, n, f) != n) die("%s: short read", path.c_str());
    fclose(f);
    el.src.resize(n);
    el.dst.resize(n);
    for (size_t i = 0; i < n; i++) {
        el.src[i] = raw[2 * i];
        el.dst[i] = raw[2 * i + 1];
        if (el.src[i] == 0xffffffffu || el.dst[i] == 0xffffffffu)
            die("%s: pair %llu: vertex id 4294967295 leaves no room for V", path.c_str(), (unsigned long long)i);
    }
}

uint64_t splitmix(uint64_t x) {
    x += 0x9e3779b97f4a7c15ull;
    x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
    x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
    return x ^ (x >> 31);
}

// Stable counting sort of the edges by key (source for CSR, destination for
// CSC): ptr gets V + 1 offsets, order[k] the input index of the k-th placed edge.
void bucket(const std::vector<uint32_t> &key, uint64_t V, std::vector<uint64_t> &ptr, std::vector<uint64_t> &order) {
    ptr.assign(V + 1, 0);
    for (uint32_t k : key) ptr[k + 1]++;
    for (uint64_t v = 0; v < V; v++) ptr[v + 1] += ptr[v];
    std::vector<uint64_t> fill(ptr.begin(), ptr.end() - 1);
    order.resize(key.size());
    for (size_t i = 0; i < key.size(); i++) order[fill[key[i]]++] = i;
}

// converter.cpp:131-138: once the running offset reaches E it steps back one.
void compat_offsets(std::vector<uint64_t> &ptr, uint64_t V, uint64_t E) {
    uint64_t t = 0;
    for (uint64_t v = 0; v < V; v++) {
        const uint64_t deg = ptr[v + 1] - ptr[v];
        ptr[v] = t;
        t += deg;
        if (t == E && E) t--;
    }
}

void write(const std::string &path, asc_format fmt, uint64_t V, uint64_t E, const uint64_t *ptr, const void *edges,
           const uint32_t *outdeg) {
    asc_status s = asc_write_graph(path.c_str(), fmt, V, E, ptr, edges, outdeg);
    if (s != ASC_OK) {
        char msg[512];
        asc_last_error(msg, sizeof(msg));
        die("%s", msg);
    }
    printf("wrote %s (V=%llu E=%llu)\n", path.c_str(), (unsigned long long)V, (unsigned long long)E);
}

}  // namespace

int main(int argc, char **argv) {
    if (argc < 2 || argv[1][0] == '-') {
        fprintf(stderr,
                "usage: asc-convert INPUT [--to toB,bcsr,bwcsr,bcsc,bcsr32] [--out STEM] [--symmetrize]\n"
                "                   [--transpose] [--weights ref|uniform[:LO:HI]|column] [--seed N] [--compat]\n");
        return 1;
    }
    std::string input = argv[1], to = "bcsr,bwcsr,bcsc", stem, weights = "ref";
    bool symmetrize = false, transpose = false, compat = false;
    unsigned long long seed = 1;
    for (int i = 2; i < argc; i++) {
        const std::string k = argv[i];
        auto value = [&]() -> std::string {
            if (i + 1 >= argc) die("%s needs a value", k.c_str());
            return argv[++i];
        };
        if (k == "--to") to = value();
        else if (k == "--out") stem = value();
        else if (k == "--weights") weights = value();
        else if (k == "--seed") seed = strtoull(value().c_str(), nullptr, 10);
        else if (k == "--symmetrize") symmetrize = true;
        else if (k == "--transpose") transpose = true;
        else if (k == "--compat") compat = true;
        else die("unknown option %s", k.c_str());
    }
    if (stem.empty()) {
        const size_t slash = input.find_last_of('/'), dot = input.find_last_of('.');
        stem = (dot != std::string::npos && (slash == std::string::npos || dot > slash)) ? input.substr(0, dot) : input;
    }
    std::vector<std::string> outs;
    for (size_t b = 0; b <= to.size();) {
        size_t e = to.find(',', b);
        if (e == std::string::npos) e = to.size();
        const std::string f = to.substr(b, e - b);
        if (f != "toB" && f != "bcsr" && f != "bwcsr" && f != "bcsc" && f != "bcsr32")
            die("unknown output format '%s'", f.c_str());
        outs.push_back(f);
        b = e + 1;
    }

    EdgeList el;
    if (ends_with(input, ".toB")) read_pairs(input, el);
    else read_text(input, el);
    size_t E0 = el.src.size();

    // weights, one per input edge, drawn before any edge is added or reordered
    uint32_t lo = 1, hi = 63;
    if (weights == "column") {
        if (!el.has_column) die("--weights column needs a third column in %s", input.c_str());
    } else if (weights == "ref") {
        srand(0);
        el.w.resize(E0);
        for (size_t i = 0; i < E0; i++) el.w[i] = (uint32_t)(rand() % 20);
    } else if (weights.compare(0, 7, "uniform") == 0) {
        if (weights.size() > 7) {
            unsigned a, b;
            if (sscanf(weights.c_str() + 7, ":%u:%u", &a, &b) != 2 || a > b) die("bad --weights %s", weights.c_str());
            lo = a;
            hi = b;
        }
        el.w.resize(E0);
        for (size_t i = 0; i < E0; i++)
            el.w[i] = lo + (uint32_t)(splitmix(seed * 0x100000001b3ull ^ i) % ((uint64_t)hi - lo + 1));
    } else {
        die("unknown --weights %s", weights.c_str());
    }
    if (transpose) std::swap(el.src, el.dst);
    if (symmetrize) {
        el.src.reserve(2 * E0);
        el.dst.reserve(2 * E0);
        el.w.reserve(2 * E0);
        for (size_t i = 0; i < E0; i++) {
            el.src.push_back(el.dst[i]);
            el.dst.push_back(el.src[i]);
            el.w.push_back(el.w[i]);
        }
    }
    const uint64_t E = el.src.size();
    uint64_t V = 0;
    for (uint64_t i = 0; i < E; i++) V = std::max<uint64_t>(V, std::max(el.src[i], el.dst[i]) + 1ull);

    for (const std::string &f : outs) {
        const std::string path = stem + "." + f;
        if (f == "toB") {
            std::vector<uint32_t> raw(2 * E);
            for (uint64_t i = 0; i < E; i++) {
                raw[2 * i] = el.src[i];
                raw[2 * i + 1] = el.dst[i];
            }
            FILE *o = fopen(path.c_str(), "wb");
            if (!o || (E && fwrite(raw.data(), 8, E, o) != E) || fclose(o) != 0) die("%s: write failed", path.c_str());
            printf("wrote %s (E=%llu)\n", path.c_str(), (unsigned long long)E);
            continue;
        }
        const bool csc = f == "bcsc";
        std::vector<uint64_t> ptr, order;
        bucket(csc ? el.dst : el.src, V, ptr, order);
        std::vector<uint32_t> outdeg;
        if (csc) {
            outdeg.assign(V, 0);
            for (uint32_t s : el.src) outdeg[s]++;
        }
        if (compat) compat_offsets(ptr, V, E);
        if (f == "bwcsr") {
            std::vector<uint32_t> ew(2 * E);
            for (uint64_t k = 0; k < E; k++) {
                ew[2 * k] = el.dst[order[k]];
                ew[2 * k + 1] = el.w[order[k]];
            }
            write(path, ASC_FMT_BWCSR, V, E, ptr.data(), ew.data(), nullptr);
        } else {
            std::vector<uint32_t> col(E);
            for (uint64_t k = 0; k < E; k++) col[k] = csc ? el.src[order[k]] : el.dst[order[k]];
            write(path, csc ? ASC_FMT_BCSC : (f == "bcsr32" ? ASC_FMT_BCSR32 : ASC_FMT_BCSR), V, E, ptr.data(),
                  col.data(), csc ? outdeg.data() : nullptr);
        }
    }
    return 0;
}
