// Point and mesh file I/O.
// Input formats follow the reference's PointStream family (PointStream.inl):
// PLY with a 'vertex' element carrying x,y,z,nx,ny,nz (ascii or binary, either
// byte order, any numeric property type), '.bnpts' raw float32 sextuples, and
// anything else as whitespace-separated ascii sextuples.  Output is a triangle
// PLY (PlyWriteTriangles, plyfile.cu:2769-2836): float x,y,z per vertex and a
// 'vertex_indices' list per face, ascii or binary little endian.
//
// The reference reads a PLY element by element through plyfile's per-property
// callbacks (PointStream.inl:227-239) and writes ascii with one fprintf per
// vertex and face.  Here the file is memory-mapped and split across host
// threads: binary vertex records of fixed size are converted in parallel ranges,
// ascii vertex lines are parsed in parallel once every line is known to hold one
// record (else the sequential parser reads the file), and ascii output is
// formatted in parallel chunks written in order -- the same bytes as a
// sequential writer.
#include <fcntl.h>
#include <sys/mman.h>
#include <sys/stat.h>
#include <unistd.h>

#include <algorithm>
#include <atomic>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "../../include/prgpu.h"

namespace prgpu {
void set_last_error(const char* fmt, ...);
}

namespace {

std::vector<float> g_xyz, g_nrm;

// ---- host threads over index ranges
int io_threads(int64_t n, int64_t min_per_thread) {
    unsigned hw = std::thread::hardware_concurrency();
    int64_t t = hw ? (int64_t)hw : 1;
    t = std::min<int64_t>(t, 64);
    t = std::min<int64_t>(t, std::max<int64_t>(1, n / std::max<int64_t>(min_per_thread, 1)));
    return (int)std::max<int64_t>(t, 1);
}

// f(lo, hi, part) over nparts contiguous ranges of [0, n)
template <class F>
void parallel_parts(int64_t n, int nparts, F&& f) {
    if (nparts <= 1) {
        f((int64_t)0, n, 0);
        return;
    }
    std::vector<std::thread> th;
    th.reserve(nparts);
    for (int k = 0; k < nparts; ++k) {
        const int64_t lo = n * k / nparts, hi = n * (k + 1) / nparts;
        th.emplace_back([&f, lo, hi, k]() { f(lo, hi, k); });
    }
    for (auto& t : th) t.join();
}

// ---- read-only mapping of a whole file
struct Mapped {
    const unsigned char* p = nullptr;
    size_t n = 0;
    void* base = nullptr;
    int fd = -1;
    bool open(const char* path) {
        fd = ::open(path, O_RDONLY);
        if (fd < 0) return false;
        struct stat st;
        if (fstat(fd, &st) != 0) return false;
        n = (size_t)st.st_size;
        if (n == 0) return true;
        base = mmap(nullptr, n, PROT_READ, MAP_PRIVATE, fd, 0);
        if (base == MAP_FAILED) {
            base = nullptr;
            return false;
        }
        p = (const unsigned char*)base;
        return true;
    }
    ~Mapped() {
        if (base) munmap(base, n);
        if (fd >= 0) ::close(fd);
    }
};

// ---- PLY property types
enum Ty { T_NONE, T_I8, T_U8, T_I16, T_U16, T_I32, T_U32, T_F32, T_F64 };

Ty type_of(const std::string& t) {
    if (t == "char" || t == "int8") return T_I8;
    if (t == "uchar" || t == "uint8") return T_U8;
    if (t == "short" || t == "int16") return T_I16;
    if (t == "ushort" || t == "uint16") return T_U16;
    if (t == "int" || t == "int32") return T_I32;
    if (t == "uint" || t == "uint32") return T_U32;
    if (t == "float" || t == "float32") return T_F32;
    if (t == "double" || t == "float64") return T_F64;
    return T_NONE;
}

int ty_size(Ty t) {
    switch (t) {
        case T_I8: case T_U8: return 1;
        case T_I16: case T_U16: return 2;
        case T_I32: case T_U32: case T_F32: return 4;
        case T_F64: return 8;
        default: return 0;
    }
}

// value of a binary property, through double as the sequential reader converts it
double load_binary(const unsigned char* p, Ty t, bool swap) {
    unsigned char b[8];
    const int n = ty_size(t);
    for (int i = 0; i < n; ++i) b[i] = swap ? p[n - 1 - i] : p[i];
    switch (t) {
        case T_I8: return (double)(int8_t)b[0];
        case T_U8: return (double)b[0];
        case T_I16: { int16_t v; memcpy(&v, b, 2); return v; }
        case T_U16: { uint16_t v; memcpy(&v, b, 2); return v; }
        case T_I32: { int32_t v; memcpy(&v, b, 4); return v; }
        case T_U32: { uint32_t v; memcpy(&v, b, 4); return v; }
        case T_F32: { float v; memcpy(&v, b, 4); return v; }
        default: { double v; memcpy(&v, b, 8); return v; }
    }
}

bool host_little_endian() {
    uint16_t v = 1;
    unsigned char c;
    memcpy(&c, &v, 1);
    return c == 1;
}

struct Prop {
    std::string name;
    Ty type = T_NONE, count_type = T_NONE;
    bool list = false;
};
struct Elem {
    std::string name;
    long long count = 0;
    std::vector<Prop> props;
    bool fixed() const {
        for (auto& p : props)
            if (p.list || p.type == T_NONE) return false;
        return true;
    }
    int64_t record_size() const {
        int64_t s = 0;
        for (auto& p : props) s += ty_size(p.type);
        return s;
    }
};

struct Header {
    int fmt = -1;   // 0 ascii, 1 binary le, 2 binary be
    std::vector<Elem> elems;
    size_t data = 0;   // first byte after end_header
};

bool parse_header(const unsigned char* d, size_t n, const char* path, Header& h) {
    size_t pos = 0;
    auto getline = [&](std::string& line) -> bool {
        if (pos >= n) return false;
        size_t e = pos;
        while (e < n && d[e] != '\n') ++e;
        line.assign((const char*)d + pos, e - pos);
        if (!line.empty() && line.back() == '\r') line.pop_back();
        pos = e + 1;
        return true;
    };
    std::string line;
    if (!getline(line) || line != "ply") {
        prgpu::set_last_error("%s: not a PLY file", path);
        return false;
    }
    bool ended = false;
    while (getline(line)) {
        char w0[64] = {0}, w1[64] = {0}, w2[64] = {0}, w3[64] = {0}, w4[64] = {0};
        int nw = sscanf(line.c_str(), "%63s %63s %63s %63s %63s", w0, w1, w2, w3, w4);
        if (nw <= 0) continue;
        std::string k = w0;
        if (k == "format") {
            std::string t = w1;
            h.fmt = (t == "ascii") ? 0 : (t == "binary_little_endian") ? 1 : (t == "binary_big_endian") ? 2 : -1;
        } else if (k == "element") {
            Elem e;
            e.name = w1;
            e.count = atoll(w2);
            h.elems.push_back(e);
        } else if (k == "property" && !h.elems.empty()) {
            Prop p;
            if (std::string(w1) == "list") {
                p.list = true;
                p.count_type = type_of(w2);
                p.type = type_of(w3);
                p.name = w4;
            } else {
                p.type = type_of(w1);
                p.name = w2;
            }
            h.elems.back().props.push_back(p);
        } else if (k == "end_header") {
            ended = true;
            break;
        }
    }
    if (!ended || h.fmt < 0) {
        prgpu::set_last_error("%s: unsupported PLY format", path);
        return false;
    }
    h.data = pos;
    return true;
}

const char* const kWant[6] = {"x", "y", "z", "nx", "ny", "nz"};

bool vertex_columns(const Elem& e, const char* path, int col[6]) {
    for (int w = 0; w < 6; ++w) col[w] = -1;
    for (size_t i = 0; i < e.props.size(); ++i)
        for (int w = 0; w < 6; ++w)
            if (e.props[i].name == kWant[w] && !e.props[i].list) col[w] = (int)i;
    for (int w = 0; w < 6; ++w)
        if (col[w] < 0) {
            prgpu::set_last_error("%s: vertex lacks %s", path, kWant[w]);
            return false;
        }
    return true;
}

// ---- sequential reader: any element order, list properties anywhere
int read_ply_sequential(const unsigned char* data, size_t n, const Header& h, const char* path) {
    size_t pos = h.data;
    const int fmt = h.fmt;
    g_xyz.clear();
    g_nrm.clear();
    const bool swap = (fmt == 1) != host_little_endian();
    for (auto& e : h.elems) {
        int col[6] = {-1, -1, -1, -1, -1, -1};
        const bool is_vertex = e.name == "vertex";
        if (is_vertex) {
            if (!vertex_columns(e, path, col)) return PRGPU_ERR_IO;
            g_xyz.resize(3 * e.count);
            g_nrm.resize(3 * e.count);
        }
        for (long long r = 0; r < e.count; ++r) {
            double v[64];
            for (size_t i = 0; i < e.props.size(); ++i) {
                const Prop& p = e.props[i];
                if (fmt == 0) {
                    while (pos < n && isspace(data[pos])) ++pos;
                    if (pos >= n) { prgpu::set_last_error("%s: truncated", path); return PRGPU_ERR_IO; }
                    char* end = nullptr;
                    const char* at = (const char*)data + pos;
                    double x = strtod(at, &end);
                    if (end == at) { prgpu::set_last_error("%s: bad number", path); return PRGPU_ERR_IO; }
                    pos = end - (const char*)data;
                    if (p.list) {
                        for (long long q = 0; q < (long long)x; ++q) {
                            while (pos < n && isspace(data[pos])) ++pos;
                            strtod((const char*)data + pos, &end);
                            pos = end - (const char*)data;
                        }
                    } else if (i < 64) {
                        v[i] = x;
                    }
                } else {
                    if (p.list) {
                        const int cs = ty_size(p.count_type), es = ty_size(p.type);
                        if (!cs || !es || pos + cs > n) { prgpu::set_last_error("%s: truncated", path); return PRGPU_ERR_IO; }
                        const long long cnt = (long long)load_binary(&data[pos], p.count_type, swap);
                        pos += cs + (size_t)(cnt * es);
                    } else {
                        const int ts = ty_size(p.type);
                        if (!ts || pos + ts > n) { prgpu::set_last_error("%s: truncated", path); return PRGPU_ERR_IO; }
                        if (i < 64) v[i] = load_binary(&data[pos], p.type, swap);
                        pos += ts;
                    }
                }
            }
            if (is_vertex) {
                for (int w = 0; w < 3; ++w) {
                    g_xyz[3 * r + w] = (float)v[col[w]];
                    g_nrm[3 * r + w] = (float)v[col[3 + w]];
                }
            }
        }
        if (is_vertex) break;
    }
    if (g_xyz.empty()) { prgpu::set_last_error("%s: no vertices", path); return PRGPU_ERR_IO; }
    return PRGPU_OK;
}

// ---- binary fast path: fixed-size records before and in the vertex element
// returns 1 when it read the points, 0 when the layout needs the sequential reader
int read_ply_binary_parallel(const unsigned char* data, size_t n, const Header& h, const char* path, int& rc) {
    size_t pos = h.data;
    for (auto& e : h.elems) {
        if (!e.fixed()) return 0;
        const int64_t rs = e.record_size();
        if (e.name != "vertex") {
            pos += (size_t)(rs * e.count);
            continue;
        }
        int col[6];
        if (!vertex_columns(e, path, col)) { rc = PRGPU_ERR_IO; return 1; }
        if (e.count <= 0) return 0;
        if (pos + (size_t)(rs * e.count) > n) { prgpu::set_last_error("%s: truncated", path); rc = PRGPU_ERR_IO; return 1; }
        int64_t off[6];
        Ty ty[6];
        for (int w = 0; w < 6; ++w) {
            off[w] = 0;
            for (int i = 0; i < col[w]; ++i) off[w] += ty_size(e.props[i].type);
            ty[w] = e.props[col[w]].type;
        }
        const bool swap = (h.fmt == 1) != host_little_endian();
        g_xyz.resize(3 * e.count);
        g_nrm.resize(3 * e.count);
        const unsigned char* base = data + pos;
        float* xyz = g_xyz.data();
        float* nrm = g_nrm.data();
        parallel_parts(e.count, io_threads(e.count, 1 << 16), [&](int64_t lo, int64_t hi, int) {
            for (int64_t r = lo; r < hi; ++r) {
                const unsigned char* rec = base + r * rs;
                for (int w = 0; w < 3; ++w) {
                    xyz[3 * r + w] = (float)load_binary(rec + off[w], ty[w], swap);
                    nrm[3 * r + w] = (float)load_binary(rec + off[3 + w], ty[3 + w], swap);
                }
            }
        });
        rc = PRGPU_OK;
        return 1;
    }
    return 0;
}

// ---- ascii fast path: 'vertex' is the first element, one record per line
int read_ply_ascii_parallel(const unsigned char* data, size_t n, const Header& h, const char* path, int& rc) {
    if (h.elems.empty() || h.elems[0].name != "vertex") return 0;
    const Elem& e = h.elems[0];
    if (!e.fixed() || e.count <= 0 || e.props.size() > 64) return 0;
    int col[6];
    if (!vertex_columns(e, path, col)) { rc = PRGPU_ERR_IO; return 1; }
    const int np = (int)e.props.size();
    const char* s = (const char*)data + h.data;
    const char* end = (const char*)data + n;
    const int64_t bytes = end - s;
    if (bytes <= 0) return 0;
    const int parts = io_threads(bytes, 1 << 20);
    // newlines per part, then the index of the first line that starts in each part
    std::vector<int64_t> nl(parts, 0);
    parallel_parts(bytes, parts, [&](int64_t lo, int64_t hi, int k) {
        int64_t c = 0;
        for (int64_t i = lo; i < hi; ++i) c += s[i] == '\n';
        nl[k] = c;
    });
    std::vector<int64_t> before(parts, 0);
    for (int k = 1; k < parts; ++k) before[k] = before[k - 1] + nl[k - 1];
    g_xyz.resize(3 * e.count);
    g_nrm.resize(3 * e.count);
    float* xyz = g_xyz.data();
    float* nrm = g_nrm.data();
    std::atomic<bool> bad(false);
    std::atomic<int64_t> got(0);
    parallel_parts(bytes, parts, [&](int64_t lo, int64_t hi, int k) {
        // first line start at or after lo: s, or the byte after a newline at index >= lo - 1
        int64_t i = lo, line = before[k];
        if (lo > 0) {
            int64_t q = lo - 1;
            while (q < bytes && s[q] != '\n') ++q;
            i = q + 1;
            if (q >= lo) ++line;   // that newline lies in this part
        }
        int64_t mine = 0;
        double v[64];
        while (i < hi && i < bytes && line < e.count && !bad.load(std::memory_order_relaxed)) {
            const char* p = s + i;
            for (int q = 0; q < np; ++q) {
                while (p < end && (*p == ' ' || *p == '\t')) ++p;
                if (p >= end || *p == '\n' || *p == '\r') { bad = true; return; }
                char* stop = nullptr;
                v[q] = strtod(p, &stop);
                if (stop == p) { bad = true; return; }
                p = stop;
            }
            while (p < end && (*p == ' ' || *p == '\t' || *p == '\r')) ++p;
            if (p < end && *p != '\n') { bad = true; return; }   // more than one record on the line
            for (int w = 0; w < 3; ++w) {
                xyz[3 * line + w] = (float)v[col[w]];
                nrm[3 * line + w] = (float)v[col[3 + w]];
            }
            ++mine;
            ++line;
            i = (p - s) + 1;
        }
        got += mine;
    });
    if (bad || got.load() != e.count) return 0;   // blank lines or several records per line
    rc = PRGPU_OK;
    return 1;
}

int read_ply(const char* path) {
    Mapped m;
    if (!m.open(path)) { prgpu::set_last_error("cannot open %s", path); return PRGPU_ERR_IO; }
    Header h;
    if (!parse_header(m.p, m.n, path, h)) return PRGPU_ERR_IO;
    int rc = PRGPU_OK;
    if (h.fmt == 0 ? read_ply_ascii_parallel(m.p, m.n, h, path, rc) : read_ply_binary_parallel(m.p, m.n, h, path, rc))
        return rc;
    return read_ply_sequential(m.p, m.n, h, path);
}

}  // namespace

extern "C" {

int prgpu_read_points(const char* path, int64_t* n, const float** xyz, const float** nrm) {
    if (!path || !n || !xyz || !nrm) return PRGPU_ERR_ARG;
    std::string p(path);
    std::string ext = p.size() >= 4 ? p.substr(p.size() - 4) : "";
    for (auto& ch : ext) ch = (char)tolower(ch);
    int rc = PRGPU_OK;
    if (ext == ".ply") {
        rc = read_ply(path);
    } else {
        std::string e6 = p.size() >= 6 ? p.substr(p.size() - 6) : "";
        g_xyz.clear();
        g_nrm.clear();
        if (e6 == ".bnpts") {
            Mapped m;
            if (!m.open(path)) { prgpu::set_last_error("cannot open %s", path); return PRGPU_ERR_IO; }
            const int64_t cnt = (int64_t)(m.n / (6 * sizeof(float)));
            g_xyz.resize(3 * cnt);
            g_nrm.resize(3 * cnt);
            const unsigned char* base = m.p;
            float* x = g_xyz.data();
            float* nv = g_nrm.data();
            parallel_parts(cnt, io_threads(cnt, 1 << 16), [&](int64_t lo, int64_t hi, int) {
                for (int64_t r = lo; r < hi; ++r) {
                    float b[6];
                    memcpy(b, base + r * 6 * sizeof(float), sizeof b);
                    for (int w = 0; w < 3; ++w) { x[3 * r + w] = b[w]; nv[3 * r + w] = b[3 + w]; }
                }
            });
        } else {
            FILE* f = fopen(path, "rb");
            if (!f) { prgpu::set_last_error("cannot open %s", path); return PRGPU_ERR_IO; }
            float b[6];
            while (fscanf(f, " %f %f %f %f %f %f ", &b[0], &b[1], &b[2], &b[3], &b[4], &b[5]) == 6)
                for (int w = 0; w < 3; ++w) { g_xyz.push_back(b[w]); g_nrm.push_back(b[3 + w]); }
            fclose(f);
        }
        if (g_xyz.empty()) { prgpu::set_last_error("%s: no points", path); rc = PRGPU_ERR_IO; }
    }
    if (rc) return rc;
    *n = (int64_t)g_xyz.size() / 3;
    *xyz = g_xyz.data();
    *nrm = g_nrm.data();
    return PRGPU_OK;
}

int prgpu_write_mesh_ply(const char* path, const prgpu_mesh* m, int32_t binary) {
    if (!path || !m) return PRGPU_ERR_ARG;
    if (binary && !host_little_endian()) { prgpu::set_last_error("big-endian host"); return PRGPU_ERR_IO; }
    FILE* f = fopen(path, "wb");
    if (!f) { prgpu::set_last_error("cannot write %s", path); return PRGPU_ERR_IO; }
    fprintf(f, "ply\nformat %s 1.0\nelement vertex %lld\nproperty float x\nproperty float y\nproperty float z\n"
               "element face %lld\nproperty list uchar int vertex_indices\nend_header\n",
            binary ? "binary_little_endian" : "ascii", (long long)m->n_vertices, (long long)m->n_triangles);
    const int64_t nv = m->n_vertices, nt = m->n_triangles;
    if (binary) {
        fwrite(m->vertices, sizeof(float), (size_t)(3 * nv), f);
        std::vector<unsigned char> buf((size_t)nt * 13);
        unsigned char* b = buf.data();
        const int32_t* tri = m->triangles;
        parallel_parts(nt, io_threads(nt, 1 << 18), [&](int64_t lo, int64_t hi, int) {
            for (int64_t t = lo; t < hi; ++t) {
                b[13 * t] = 3;
                memcpy(&b[13 * t + 1], &tri[3 * t], 12);
            }
        });
        fwrite(buf.data(), 1, buf.size(), f);
    } else {
        // parts formatted in parallel, written in order
        auto emit = [&](int64_t count, auto&& line) {
            const int parts = io_threads(count, 1 << 16);
            std::vector<std::string> out(parts);
            parallel_parts(count, parts, [&](int64_t lo, int64_t hi, int k) {
                std::string& s = out[k];
                s.reserve((size_t)(hi - lo) * 32);
                char tmp[128];
                for (int64_t i = lo; i < hi; ++i) {
                    const int len = line(tmp, sizeof tmp, i);
                    s.append(tmp, (size_t)len);
                }
            });
            for (auto& s : out) fwrite(s.data(), 1, s.size(), f);
        };
        const float* v = m->vertices;
        const int32_t* t = m->triangles;
        emit(nv, [v](char* b, size_t cap, int64_t i) {
            return snprintf(b, cap, "%g %g %g\n", v[3 * i], v[3 * i + 1], v[3 * i + 2]);
        });
        emit(nt, [t](char* b, size_t cap, int64_t i) {
            return snprintf(b, cap, "3 %d %d %d\n", t[3 * i], t[3 * i + 1], t[3 * i + 2]);
        });
    }
    int bad = ferror(f);
    fclose(f);
    return bad ? PRGPU_ERR_IO : PRGPU_OK;
}

}  // extern "C"
