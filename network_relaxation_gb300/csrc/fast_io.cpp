/*
 * Network files at scale: parallel .dat and .nmc readers with the
 * reference's exact line semantics (read_network, large_strain_relax.cu:
 * 42-114; read_network_mesh, network_mesh_relax.cu:72-230), parallel
 * writers, and a binary side-car that also keeps the triples.
 *
 * Reader.  The reference reads line by line with std::getline / eof() and
 * sscanf.  Here the file is read at once and cut into the same lines (a
 * line ends at '\n'; reading the segment after the last '\n' is what sets
 * eof; sscanf sees a line only up to its first NUL), every line is parsed
 * in parallel both as a point ("%lf %lf") and as a bond ("%d %d %hhd"),
 * and the reference's sequential state machine then runs over the parsed
 * lines.  Tokens of the plain decimal form are converted with
 * std::from_chars (correctly rounded, like glibc's strtod that sscanf
 * uses); a line with any other token is handed to sscanf itself, so every
 * line gives exactly sscanf's result.
 *
 * Threads: NR_IO_THREADS, default std::thread::hardware_concurrency().
 * Compiled with -ffp-contract=off (rest lengths as the reference computes
 * them).
 */
#include <algorithm>
#include <cfloat>
#include <charconv>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "nr_internal.h"

namespace nr {
namespace {

int io_threads() {
    const char *env = getenv("NR_IO_THREADS");
    int t = env ? atoi(env) : 0;
    if (t <= 0) t = (int)std::thread::hardware_concurrency();
    return std::max(1, std::min(t, 256));
}

/* Runs f(begin, end) over [0, n) in contiguous chunks on up to `threads`
 * threads (the calling thread takes the first chunk). */
template <class F>
void parallel_ranges(long n, int threads, F &&f) {
    const long min_chunk = 4096;
    const int t = (int)std::max(1L, std::min<long>(threads, (n + min_chunk - 1) / min_chunk));
    if (t <= 1) {
        f(0L, n);
        return;
    }
    std::vector<std::thread> pool;
    const long per = (n + t - 1) / t;
    for (int k = 1; k < t; ++k) {
        const long b = std::min(n, k * per), e = std::min(n, (k + 1) * per);
        pool.emplace_back([=, &f] { f(b, e); });
    }
    f(0L, std::min(n, per));
    for (auto &th : pool) th.join();
}

inline bool is_space(char c) { return c == ' ' || c == '\t' || c == '\n' || c == '\v' || c == '\f' || c == '\r'; }

/* A plain decimal real: [+-]? (digits [. digits*] | . digits) ([eE] [+-]? digits)?,
 * ending at whitespace or at the end of the line. */
bool strict_double(const char *&p, const char *e, double &v) {
    const char *q = p;
    const char *start = p;
    if (q < e && (*q == '+' || *q == '-')) ++q;
    const char *num = (*start == '+') ? start + 1 : start;
    int digits = 0;
    while (q < e && *q >= '0' && *q <= '9') ++q, ++digits;
    if (q < e && *q == '.') {
        ++q;
        while (q < e && *q >= '0' && *q <= '9') ++q, ++digits;
    }
    if (digits == 0) return false;
    if (q < e && (*q == 'e' || *q == 'E')) {
        ++q;
        if (q < e && (*q == '+' || *q == '-')) ++q;
        int ed = 0;
        while (q < e && *q >= '0' && *q <= '9') ++q, ++ed;
        if (ed == 0) return false;
    }
    if (q < e && !is_space(*q)) return false;
    if (q - start > 400) return false;
    auto r = std::from_chars(num, q, v, std::chars_format::general);
    if (r.ec != std::errc() || r.ptr != q) return false;
    p = q;
    return true;
}

/* A plain decimal integer of at most 9 digits, ending at whitespace or at the
 * end of the line. */
bool strict_int(const char *&p, const char *e, long &v) {
    const char *q = p;
    bool neg = false;
    if (q < e && (*q == '+' || *q == '-')) neg = *q++ == '-';
    long acc = 0;
    int digits = 0;
    while (q < e && *q >= '0' && *q <= '9') {
        acc = acc * 10 + (*q++ - '0');
        if (++digits > 9) return false;
    }
    if (digits == 0 || (q < e && !is_space(*q))) return false;
    v = neg ? -acc : acc;
    p = q;
    return true;
}

inline void skip_space(const char *&p, const char *e) {
    while (p < e && is_space(*p)) ++p;
}

struct PointLine {
    double x, y;
    int n;
};
struct EdgeLine {
    int i1, i2;
    signed char mult;
    int n;
};

/* sscanf(line, "%lf %lf", ...) */
PointLine parse_point(const char *b, const char *e) {
    PointLine r{0, 0, 0};
    const char *p = b;
    skip_space(p, e);
    if (p == e) {
        r.n = -1;
        return r;
    }
    if (strict_double(p, e, r.x)) {
        r.n = 1;
        skip_space(p, e);
        if (p == e) return r;
        if (strict_double(p, e, r.y)) {
            r.n = 2;
            return r;
        }
    }
    const std::string line(b, e);
    r.n = sscanf(line.c_str(), "%lf %lf", &r.x, &r.y);
    return r;
}

/* sscanf(line, "%d %d %hhd\n", ...) */
EdgeLine parse_edge(const char *b, const char *e) {
    EdgeLine r{0, 0, 0, 0};
    const char *p = b;
    skip_space(p, e);
    if (p == e) {
        r.n = -1;
        return r;
    }
    long v1, v2, v3;
    if (strict_int(p, e, v1)) {
        r.i1 = (int)v1;
        r.n = 1;
        skip_space(p, e);
        if (p == e) return r;
        if (strict_int(p, e, v2)) {
            r.i2 = (int)v2;
            r.n = 2;
            skip_space(p, e);
            if (p == e) return r;
            if (strict_int(p, e, v3) && v3 >= -128 && v3 <= 127) {
                r.mult = (signed char)v3;
                r.n = 3;
                return r;
            }
        }
    }
    const std::string line(b, e);
    int i1 = 0, i2 = 0;
    signed char m = 0;
    r.n = sscanf(line.c_str(), "%d %d %hhd\n", &i1, &i2, &m);
    r.i1 = i1;
    r.i2 = i2;
    r.mult = m;
    return r;
}

struct FacetLine {
    int i1, i2, i3;
    int n;
};

/* sscanf(line, "%d %d %d\n", ...) */
FacetLine parse_facet(const char *b, const char *e) {
    FacetLine r{0, 0, 0, 0};
    const char *p = b;
    skip_space(p, e);
    if (p == e) {
        r.n = -1;
        return r;
    }
    long v[3];
    int k = 0;
    while (k < 3 && strict_int(p, e, v[k])) {
        ++k;
        skip_space(p, e);
        if (p == e) break;
    }
    if (k == 3 || p == e) {
        r.n = k;
        r.i1 = k > 0 ? (int)v[0] : 0;
        r.i2 = k > 1 ? (int)v[1] : 0;
        r.i3 = k > 2 ? (int)v[2] : 0;
        return r;
    }
    const std::string line(b, e);
    r.n = sscanf(line.c_str(), "%d %d %d\n", &r.i1, &r.i2, &r.i3);
    return r;
}

/* The file cut into std::getline's lines; the last line is the one whose
 * reading sets eof.  end points at the first NUL of a line (sscanf's view). */
struct Lines {
    std::vector<char> buf;
    std::vector<const char *> begin, end;
    bool load(const char *path) {
        FILE *f = fopen(path, "rb");
        if (!f) return false;
        fseek(f, 0, SEEK_END);
        const long size = ftell(f);
        fseek(f, 0, SEEK_SET);
        buf.resize(size > 0 ? (size_t)size : 0);
        const size_t got = size > 0 ? fread(buf.data(), 1, (size_t)size, f) : 0;
        fclose(f);
        buf.resize(got);
        buf.push_back('\0'); /* a valid address for an empty file; not part of any line */
        const char *p = buf.data(), *e = buf.data() + got;
        for (;;) {
            const char *nl = (const char *)memchr(p, '\n', (size_t)(e - p));
            const char *le = nl ? nl : e;
            const char *z = (const char *)memchr(p, '\0', (size_t)(le - p));
            begin.push_back(p);
            end.push_back(z ? z : le);
            if (!nl) break;
            p = nl + 1;
        }
        return true;
    }
    size_t count() const { return begin.size(); }
};

}  // namespace
}  // namespace nr

using nr::fail;

extern "C" {

/* read_network, large_strain_relax.cu:42-114 (see the file comment). */
int nr_read_network(const char *path, nr_host_network **out) {
    if (!path || !out) return fail(NR_ERR_INVALID, "nr_read_network: null argument");
    *out = nullptr;
    nr::Lines L;
    if (!L.load(path)) return fail(NR_ERR_IO, std::string("cannot open ") + path);
    auto *net = new nr_host_network();
    *out = net;
    const size_t nl = L.count();
    size_t cur = 0; /* next line to read */
    auto eof_after = [&](size_t line) { return line + 1 >= nl; };
    int num_points = 0, num_edges = 0;
    double offset = 0;
    net->miny = FLT_MAX;
    net->maxy = FLT_MIN;
    {
        const std::string header(L.begin[0], L.end[0]);
        const int num_read = sscanf(header.c_str(), "%d %d %lf", &num_points, &num_edges, &offset);
        cur = 1;
        if (num_read < 3 || offset < 0 || num_points <= 0 || num_edges < 0)
            return fail(NR_ERR_PARSE, "Reading failed. The provided file has an invalid header.");
    }
    net->offset = offset;
    bool eof = eof_after(0);
    const int threads = nr::io_threads();
    /* parse every remaining line both ways, in parallel */
    const long rest = (long)(nl - cur);
    std::vector<nr::PointLine> pl(rest);
    std::vector<nr::EdgeLine> el(rest);
    nr::parallel_ranges(rest, threads, [&](long b, long e) {
        for (long i = b; i < e; ++i) {
            pl[i] = nr::parse_point(L.begin[cur + i], L.end[cur + i]);
            el[i] = nr::parse_edge(L.begin[cur + i], L.end[cur + i]);
        }
    });
    net->points.reserve(2 * (size_t)num_points);
    while (!eof && net->points.size() < 2 * (size_t)num_points) {
        const nr::PointLine &r = pl[cur - 1];
        eof = eof_after(cur);
        ++cur;
        if (r.n == 2) {
            net->points.push_back(r.x);
            net->points.push_back(r.y);
            if (r.y < net->miny) net->miny = r.y;
            if (r.y > net->maxy) net->maxy = r.y;
        }
    }
    net->n_points = (int)(net->points.size() / 2);
    if (eof) return fail(NR_ERR_PARSE, "Reading failed. Too few points were read.");
    net->edge_ij.reserve(2 * (size_t)num_edges);
    net->edge_wrap.reserve(num_edges);
    while (!eof && net->edge_wrap.size() < (size_t)num_edges) {
        const nr::EdgeLine &r = el[cur - 1];
        eof = eof_after(cur);
        ++cur;
        if (r.n == 3) {
            if (std::min(r.i1, r.i2) > -1 && std::max(r.i1, r.i2) < num_points) {
                net->edge_ij.push_back(r.i1);
                net->edge_ij.push_back(r.i2);
                net->edge_wrap.push_back(r.mult);
            } else {
                /* l0 of the bonds read so far, then the reference's error */
                break;
            }
        }
    }
    const size_t ne = net->edge_wrap.size();
    net->edge_l0.resize(ne);
    const double *p = net->points.data();
    nr::parallel_ranges((long)ne, threads, [&](long b, long e) {
        for (long k = b; k < e; ++k) {
            const int i1 = net->edge_ij[2 * k], i2 = net->edge_ij[2 * k + 1];
            const double dx = p[2 * i2] + offset * net->edge_wrap[k] - p[2 * i1];
            const double dy = p[2 * i2 + 1] - p[2 * i1 + 1];
            net->edge_l0[k] = std::sqrt(dx * dx + dy * dy);
        }
    });
    if (ne < (size_t)num_edges) {
        const nr::EdgeLine &r = el[cur - 2 < el.size() ? cur - 2 : 0];
        const bool bad_index = cur >= 2 && r.n == 3 && !(std::min(r.i1, r.i2) > -1 && std::max(r.i1, r.i2) < num_points);
        if (bad_index) return fail(NR_ERR_PARSE, "Reading failed due to an out-of-bounds point index.");
        return fail(NR_ERR_PARSE, "Too few edges were found.");
    }
    return NR_OK;
}

/* The .dat format read_network reads (%.17g, round-trips exactly),
 * formatted in parallel with std::to_chars (whose output with a format and
 * precision is printf's), written in order. */
int nr_write_network(const nr_host_network *net, const char *path) {
    if (!net || !path) return fail(NR_ERR_INVALID, "nr_write_network: null argument");
    FILE *f = fopen(path, "w");
    if (!f) return fail(NR_ERR_IO, std::string("cannot write ") + path);
    fprintf(f, "%d %d %.17g\n", net->n_points, net->n_edges(), net->offset);
    const int threads = nr::io_threads();
    const long np = net->n_points, ne = net->n_edges();
    const int chunks = std::max(1, threads * 4);
    for (int section = 0; section < 2; ++section) {
        const long n = section == 0 ? np : ne;
        std::vector<std::string> out(chunks);
        const long per = (n + chunks - 1) / chunks;
        nr::parallel_ranges(chunks, threads, [&](long cb, long ce) {
            char line[96];
            for (long c = cb; c < ce; ++c) {
                std::string &s = out[c];
                for (long i = c * per; i < std::min(n, (c + 1) * per); ++i) {
                    char *q = line, *end = line + sizeof(line);
                    if (section == 0) {
                        q = std::to_chars(q, end, net->points[2 * i], std::chars_format::general, 17).ptr;
                        *q++ = ' ';
                        q = std::to_chars(q, end, net->points[2 * i + 1], std::chars_format::general, 17).ptr;
                    } else {
                        q = std::to_chars(q, end, net->edge_ij[2 * i]).ptr;
                        *q++ = ' ';
                        q = std::to_chars(q, end, net->edge_ij[2 * i + 1]).ptr;
                        *q++ = ' ';
                        q = std::to_chars(q, end, (int)net->edge_wrap[i]).ptr;
                    }
                    *q++ = '\n';
                    s.append(line, (size_t)(q - line));
                }
            }
        });
        for (const std::string &s : out) fwrite(s.data(), 1, s.size(), f);
    }
    const bool ok = fclose(f) == 0;
    return ok ? NR_OK : fail(NR_ERR_IO, std::string("cannot write ") + path);
}



/* read_network_mesh, network_mesh_relax.cu:72-230: header "N E F offset",
 * then points, edges "i j wrap", facets "i j k" and areas, with the
 * reference's getline / eof() / sscanf semantics (see the file comment).
 * Each line is parsed in parallel as the type its position gives it in a
 * well-formed file; the sequential state machine parses any other line it
 * meets (a junk line shifts the rest) on the spot.  On NR_ERR_PARSE the
 * partially read network is still returned. */
int nr_read_network_mesh(const char *path, nr_host_network **out) {
    if (!path || !out) return fail(NR_ERR_INVALID, "nr_read_network_mesh: null argument");
    *out = nullptr;
    nr::Lines L;
    if (!L.load(path)) return fail(NR_ERR_IO, std::string("cannot open ") + path);
    auto *net = new nr_host_network();
    *out = net;
    const size_t nl = L.count();
    auto eof_after = [&](size_t line) { return line + 1 >= nl; };
    int num_points = 0, num_edges = 0, num_facets = 0;
    double offset = 0;
    net->minx = FLT_MAX;
    net->miny = FLT_MAX;
    net->maxx = FLT_MIN;
    net->maxy = FLT_MIN;
    {
        const std::string header(L.begin[0], L.end[0]);
        const int num_read = sscanf(header.c_str(), "%d %d %d %lf", &num_points, &num_edges, &num_facets, &offset);
        if (num_read < 4 || offset < 0 || num_points <= 0 || num_edges < 0 || num_facets < 0)
            return fail(NR_ERR_PARSE, "Reading failed. The provided file has an invalid header.");
    }
    net->offset = offset;
    /* the line ranges of a well-formed file, parsed in parallel */
    const size_t lo_p = 1, lo_e = lo_p + (size_t)num_points, lo_f = lo_e + (size_t)num_edges,
                 lo_a = lo_f + (size_t)num_facets, hi = lo_a + (size_t)num_facets;
    auto clip = [&](size_t v) { return std::min(v, nl); };
    std::vector<nr::PointLine> pl(clip(lo_e) - clip(lo_p)), al(clip(hi) - clip(lo_a));
    std::vector<nr::EdgeLine> el(clip(lo_f) - clip(lo_e));
    std::vector<nr::FacetLine> fl(clip(lo_a) - clip(lo_f));
    const int threads = nr::io_threads();
    nr::parallel_ranges((long)(clip(hi) - clip(lo_p)), threads, [&](long b, long e) {
        for (long k = b; k < e; ++k) {
            const size_t li = lo_p + (size_t)k;
            if (li < lo_e) pl[li - lo_p] = nr::parse_point(L.begin[li], L.end[li]);
            else if (li < lo_f) el[li - lo_e] = nr::parse_edge(L.begin[li], L.end[li]);
            else if (li < lo_a) fl[li - lo_f] = nr::parse_facet(L.begin[li], L.end[li]);
            else al[li - lo_a] = nr::parse_point(L.begin[li], L.end[li]);
        }
    });
    auto point_at = [&](size_t li) {
        return li >= lo_p && li < lo_p + pl.size() ? pl[li - lo_p] : nr::parse_point(L.begin[li], L.end[li]);
    };
    auto area_at = [&](size_t li) {
        return li >= lo_a && li < lo_a + al.size() ? al[li - lo_a] : nr::parse_point(L.begin[li], L.end[li]);
    };
    auto edge_at = [&](size_t li) {
        return li >= lo_e && li < lo_e + el.size() ? el[li - lo_e] : nr::parse_edge(L.begin[li], L.end[li]);
    };
    auto facet_at = [&](size_t li) {
        return li >= lo_f && li < lo_f + fl.size() ? fl[li - lo_f] : nr::parse_facet(L.begin[li], L.end[li]);
    };
    size_t cur = 1;
    bool eof = eof_after(0);
    net->points.reserve(2 * (size_t)std::min<long>(num_points, (long)nl));
    while (!eof && net->points.size() < 2 * (size_t)num_points) {
        const nr::PointLine r = point_at(cur);
        eof = eof_after(cur++);
        if (r.n == 2) {
            net->points.push_back(r.x);
            net->points.push_back(r.y);
            if (r.x < net->minx) net->minx = r.x;
            if (r.y < net->miny) net->miny = r.y;
            if (r.x > net->maxx) net->maxx = r.x;
            if (r.y > net->maxy) net->maxy = r.y;
        }
    }
    net->n_points = (int)(net->points.size() / 2);
    if (eof) return fail(NR_ERR_PARSE, "Reading failed. Too few points were read.");
    bool bad_index = false;
    while (!eof && net->edge_wrap.size() < (size_t)num_edges) {
        const nr::EdgeLine r = edge_at(cur);
        eof = eof_after(cur++);
        if (r.n == 3) {
            if (std::min(r.i1, r.i2) > -1 && std::max(r.i1, r.i2) < num_points) {
                net->edge_ij.push_back(r.i1);
                net->edge_ij.push_back(r.i2);
                net->edge_wrap.push_back(r.mult);
            } else {
                bad_index = true;
                break;
            }
        }
    }
    const size_t ne = net->edge_wrap.size();
    net->edge_l0.resize(ne);
    const double *p = net->points.data();
    nr::parallel_ranges((long)ne, threads, [&](long b, long e) {
        for (long k = b; k < e; ++k) {
            const int i1 = net->edge_ij[2 * k], i2 = net->edge_ij[2 * k + 1];
            const double dx = p[2 * i2] + offset * net->edge_wrap[k] - p[2 * i1];
            const double dy = p[2 * i2 + 1] - p[2 * i1 + 1];
            net->edge_l0[k] = std::sqrt(dx * dx + dy * dy);
        }
    });
    if (bad_index) return fail(NR_ERR_PARSE, "Reading failed due to an out-of-bounds point index.");
    if (ne < (size_t)num_edges) return fail(NR_ERR_PARSE, "Too few edges were read.");
    if (eof && num_facets > 0) return fail(NR_ERR_PARSE, "The file ended before facets could be read.");
    auto in_bounds = [&](int v) { return v >= 0 && v <= num_points - 1; };
    while (!eof && net->facets.size() < 3 * (size_t)num_facets) {
        const nr::FacetLine r = facet_at(cur);
        eof = eof_after(cur++);
        if (r.n == 3) {
            if (!(in_bounds(r.i1) && in_bounds(r.i2) && in_bounds(r.i3)))
                return fail(NR_ERR_PARSE, "Reading failed due to an out-of-bounds point index.");
            net->facets.push_back(r.i1);
            net->facets.push_back(r.i2);
            net->facets.push_back(r.i3);
        }
    }
    if (net->facets.size() < 3 * (size_t)num_facets) return fail(NR_ERR_PARSE, "Too few facets were read.");
    if (eof && num_facets > 0) return fail(NR_ERR_PARSE, "The file ended before facets could be read.");
    while (!eof && net->areas.size() < (size_t)num_facets) {
        const nr::PointLine r = area_at(cur); /* sscanf("%lf") == 1: the first value parsed */
        eof = eof_after(cur++);
        if (r.n >= 1) {
            if (r.x > 0) net->areas.push_back(r.x);
            else return fail(NR_ERR_PARSE, "An illegal area was specified.");
        }
    }
    if (net->areas.size() < (size_t)num_facets) return fail(NR_ERR_PARSE, "Too few areas were specified.");
    nr::find_mesh_pairs(net->points, offset, net->minx, net->mesh_pairs);
    return NR_OK;
}

/* Writes the format nr_read_network_mesh reads (%.17g, round-trips
 * exactly), formatted in parallel like nr_write_network. */
int nr_write_network_mesh(const nr_host_network *net, const char *path) {
    if (!net || !path) return fail(NR_ERR_INVALID, "nr_write_network_mesh: null argument");
    FILE *f = fopen(path, "w");
    if (!f) return fail(NR_ERR_IO, std::string("cannot write ") + path);
    fprintf(f, "%d %d %d %.17g\n", net->n_points, net->n_edges(), net->n_facets(), net->offset);
    const int threads = nr::io_threads();
    const int chunks = std::max(1, threads * 4);
    const long counts[4] = {net->n_points, net->n_edges(), net->n_facets(), net->n_facets()};
    for (int section = 0; section < 4; ++section) {
        const long n = counts[section];
        std::vector<std::string> outs(chunks);
        const long per = (n + chunks - 1) / chunks;
        nr::parallel_ranges(chunks, threads, [&](long cb, long ce) {
            char line[128];
            for (long c = cb; c < ce; ++c) {
                for (long i = c * per; i < std::min(n, (c + 1) * per); ++i) {
                    char *q = line, *end = line + sizeof(line);
                    if (section == 0) {
                        q = std::to_chars(q, end, net->points[2 * i], std::chars_format::general, 17).ptr;
                        *q++ = ' ';
                        q = std::to_chars(q, end, net->points[2 * i + 1], std::chars_format::general, 17).ptr;
                    } else if (section == 1) {
                        q = std::to_chars(q, end, net->edge_ij[2 * i]).ptr;
                        *q++ = ' ';
                        q = std::to_chars(q, end, net->edge_ij[2 * i + 1]).ptr;
                        *q++ = ' ';
                        q = std::to_chars(q, end, (int)net->edge_wrap[i]).ptr;
                    } else if (section == 2) {
                        for (int v = 0; v < 3; ++v) {
                            if (v) *q++ = ' ';
                            q = std::to_chars(q, end, net->facets[3 * i + v]).ptr;
                        }
                    } else {
                        q = std::to_chars(q, end, net->areas[i], std::chars_format::general, 17).ptr;
                    }
                    *q++ = '\n';
                    outs[c].append(line, (size_t)(q - line));
                }
            }
        });
        for (const std::string &s : outs) fwrite(s.data(), 1, s.size(), f);
    }
    const bool ok = fclose(f) == 0;
    return ok ? NR_OK : fail(NR_ERR_IO, std::string("cannot write ") + path);
}

}  // extern "C"

namespace nr {
/* n xy pairs as the reference's report_displaced writes them
 * ("%2.10le\t%2.10le\n" per node, large_strain_relax.cu:216-227), formatted
 * in parallel (std::to_chars, scientific, 10 digits: printf's output). */
bool write_xy_file(const std::string &name, const double *xy, long n) {
    FILE *f = fopen(name.c_str(), "w");
    if (!f) return false;
    const int threads = io_threads();
    const int chunks = std::max(1, threads * 4);
    std::vector<std::string> out(chunks);
    const long per = (n + chunks - 1) / chunks;
    parallel_ranges(chunks, threads, [&](long cb, long ce) {
        char line[96];
        for (long c = cb; c < ce; ++c)
            for (long i = c * per; i < std::min(n, (c + 1) * per); ++i) {
                char *q = line, *end = line + sizeof(line);
                q = std::to_chars(q, end, xy[2 * i], std::chars_format::scientific, 10).ptr;
                *q++ = '\t';
                q = std::to_chars(q, end, xy[2 * i + 1], std::chars_format::scientific, 10).ptr;
                *q++ = '\n';
                out[c].append(line, (size_t)(q - line));
            }
    });
    for (const std::string &s : out) fwrite(s.data(), 1, s.size(), f);
    return fclose(f) == 0;
}
}  // namespace nr

extern "C" int nr_write_positions(const double *xy, int n_points, const char *path) {
    if (!xy || n_points < 0 || !path) return fail(NR_ERR_INVALID, "nr_write_positions: bad arguments");
    return nr::write_xy_file(path, xy, n_points) ? NR_OK : fail(NR_ERR_IO, std::string("cannot write ") + path);
}

/* ------------------------------------------------------ binary side-car */

namespace nr {
namespace {

constexpr char kBinMagic[8] = {'N', 'R', 'N', 'E', 'T', 'B', 'I', 'N'};
constexpr uint32_t kBinVersion = 2; /* 2: the checksum covers the header */

struct BinHeader {
    char magic[8];
    uint32_t version, flags;
    int64_t n_points, n_edges, n_triples, n_facets, n_pairs, n_areas;
    double offset, miny, maxy, minx, maxx;
    uint64_t checksum; /* FNV-1a 64 of the payload */
};

uint64_t fnv1a(uint64_t h, const void *data, size_t n) {
    const unsigned char *p = (const unsigned char *)data;
    for (size_t i = 0; i < n; ++i) {
        h ^= p[i];
        h *= 1099511628211ULL;
    }
    return h;
}

constexpr uint64_t kFnvBasis = 14695981039346656037ULL;

/* FNV-1a of the header with its checksum field zeroed: the checksum starts
 * here, so a damaged count, box or offset is caught like damaged data. */
uint64_t header_sum(const BinHeader &h) {
    BinHeader z = h;
    z.checksum = 0;
    return fnv1a(kFnvBasis, &z, sizeof(z));
}

/* Payload bytes the header announces (counts already range-checked). */
uint64_t payload_bytes(const BinHeader &h) {
    const uint64_t n = (uint64_t)h.n_points, e = (uint64_t)h.n_edges, t = (uint64_t)h.n_triples;
    uint64_t b = 16 * n + 17 * e + 14 * t + 12 * (uint64_t)h.n_facets + 8 * (uint64_t)h.n_areas +
                 8 * (uint64_t)h.n_pairs;
    if (h.flags & 1u) b += 8 * e;
    if (h.flags & 2u) b += 8 * t;
    if (h.flags & 4u) b += 8 * t;
    return b;
}

struct Payload {
    std::vector<std::pair<const void *, size_t>> parts;
    template <class T>
    void add(const std::vector<T> &v) {
        parts.push_back({v.data(), v.size() * sizeof(T)});
    }
};

}  // namespace
}  // namespace nr

extern "C" {

/* Binary copy of a host network (little-endian, as on the x86-64 and Arm
 * machines this library builds for): header, then points, bonds, rest
 * lengths, wraps, triples, optional per-item constants and the mesh, and
 * an FNV-1a checksum of it all. */
int nr_write_network_bin(const nr_host_network *net, const char *path) {
    if (!net || !path) return fail(NR_ERR_INVALID, "nr_write_network_bin: null argument");
    nr::BinHeader h;
    memset(&h, 0, sizeof(h));
    memcpy(h.magic, nr::kBinMagic, 8);
    h.version = nr::kBinVersion;
    h.flags = (net->bond_k.empty() ? 0u : 1u) | (net->tri_kb.empty() ? 0u : 2u) | (net->tri_phi0.empty() ? 0u : 4u);
    h.n_points = net->n_points;
    h.n_edges = net->n_edges();
    h.n_triples = net->n_triples();
    h.n_facets = net->n_facets();
    h.n_pairs = net->n_mesh_pairs();
    h.n_areas = (int64_t)net->areas.size();
    h.offset = net->offset;
    h.miny = net->miny;
    h.maxy = net->maxy;
    h.minx = net->minx;
    h.maxx = net->maxx;
    nr::Payload pl;
    pl.add(net->points);
    pl.add(net->edge_ij);
    pl.add(net->edge_l0);
    pl.add(net->edge_wrap);
    pl.add(net->tri_hjk);
    pl.add(net->tri_wrap);
    pl.add(net->bond_k);
    pl.add(net->tri_kb);
    pl.add(net->tri_phi0);
    pl.add(net->facets);
    pl.add(net->areas);
    pl.add(net->mesh_pairs);
    uint64_t c = nr::header_sum(h);
    for (auto &part : pl.parts) c = nr::fnv1a(c, part.first, part.second);
    h.checksum = c;
    FILE *f = fopen(path, "wb");
    if (!f) return fail(NR_ERR_IO, std::string("cannot write ") + path);
    bool ok = fwrite(&h, sizeof(h), 1, f) == 1;
    for (auto &part : pl.parts)
        if (part.second) ok = ok && fwrite(part.first, 1, part.second, f) == part.second;
    ok = (fclose(f) == 0) && ok;
    return ok ? NR_OK : fail(NR_ERR_IO, std::string("cannot write ") + path);
}

int nr_read_network_bin(const char *path, nr_host_network **out) {
    if (!path || !out) return fail(NR_ERR_INVALID, "nr_read_network_bin: null argument");
    *out = nullptr;
    FILE *f = fopen(path, "rb");
    if (!f) return fail(NR_ERR_IO, std::string("cannot open ") + path);
    nr::BinHeader h;
    if (fread(&h, sizeof(h), 1, f) != 1 || memcmp(h.magic, nr::kBinMagic, 8) != 0 || h.version != nr::kBinVersion ||
        h.n_points <= 0 || h.n_points > (1LL << 30) || h.n_edges < 0 || h.n_edges > (1LL << 31) || h.n_triples < 0 ||
        h.n_triples > (1LL << 31) || h.n_facets < 0 || h.n_facets > (1LL << 31) || h.n_pairs < 0 ||
        h.n_pairs > (1LL << 30) || h.n_areas < 0 || h.n_areas > h.n_facets || h.flags > 7u) {
        fclose(f);
        return fail(NR_ERR_PARSE, std::string("not a network binary: ") + path);
    }
    /* The file must hold exactly the announced payload: checked before
     * anything is allocated, so a damaged count cannot ask for gigabytes. */
    long here = ftell(f);
    bool size_ok = here >= 0 && fseek(f, 0, SEEK_END) == 0;
    const long end = size_ok ? ftell(f) : -1;
    size_ok = size_ok && end >= here && (uint64_t)(end - here) == nr::payload_bytes(h) && fseek(f, here, SEEK_SET) == 0;
    if (!size_ok) {
        fclose(f);
        return fail(NR_ERR_PARSE, std::string("truncated or corrupt network binary: ") + path);
    }
    auto *net = new nr_host_network();
    net->n_points = (int)h.n_points;
    net->offset = h.offset;
    net->miny = h.miny;
    net->maxy = h.maxy;
    net->minx = h.minx;
    net->maxx = h.maxx;
    net->points.resize(2 * (size_t)h.n_points);
    net->edge_ij.resize(2 * (size_t)h.n_edges);
    net->edge_l0.resize(h.n_edges);
    net->edge_wrap.resize(h.n_edges);
    net->tri_hjk.resize(3 * (size_t)h.n_triples);
    net->tri_wrap.resize(2 * (size_t)h.n_triples);
    net->bond_k.resize(h.flags & 1u ? h.n_edges : 0);
    net->tri_kb.resize(h.flags & 2u ? h.n_triples : 0);
    net->tri_phi0.resize(h.flags & 4u ? h.n_triples : 0);
    net->facets.resize(3 * (size_t)h.n_facets);
    net->areas.resize(h.n_areas);
    net->mesh_pairs.resize(2 * (size_t)h.n_pairs);
    nr::Payload pl;
    pl.add(net->points);
    pl.add(net->edge_ij);
    pl.add(net->edge_l0);
    pl.add(net->edge_wrap);
    pl.add(net->tri_hjk);
    pl.add(net->tri_wrap);
    pl.add(net->bond_k);
    pl.add(net->tri_kb);
    pl.add(net->tri_phi0);
    pl.add(net->facets);
    pl.add(net->areas);
    pl.add(net->mesh_pairs);
    bool ok = true;
    uint64_t c = nr::header_sum(h);
    for (auto &part : pl.parts) {
        if (part.second) ok = ok && fread((void *)part.first, 1, part.second, f) == part.second;
        c = nr::fnv1a(c, part.first, part.second);
    }
    fclose(f);
    if (!ok || c != h.checksum) {
        delete net;
        return fail(NR_ERR_PARSE, std::string("truncated or corrupt network binary: ") + path);
    }
    const auto in_range = [&](const std::vector<int> &v) {
        for (int x : v)
            if (x < 0 || x >= net->n_points) return false;
        return true;
    };
    if (!in_range(net->edge_ij) || !in_range(net->tri_hjk) || !in_range(net->facets) || !in_range(net->mesh_pairs)) {
        delete net;
        return fail(NR_ERR_PARSE, std::string("node index out of range in ") + path);
    }
    *out = net;
    return NR_OK;
}

}  // extern "C"
