// Point and mesh file I/O.
// Input formats follow the reference's PointStream family (PointStream.inl):
// PLY with a 'vertex' element carrying x,y,z,nx,ny,nz (ascii or binary, either
// byte order, any numeric property type), '.bnpts' raw float32 sextuples, and
// anything else as whitespace-separated ascii sextuples.  Output is a triangle
// PLY (PlyWriteTriangles, plyfile.cu:2769-2836): float x,y,z per vertex and a
// 'vertex_indices' list per face, ascii or binary little endian.
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/prgpu.h"

namespace prgpu {
void set_last_error(const char* fmt, ...);
}

namespace {

std::vector<float> g_xyz, g_nrm;

int type_size(const std::string& t) {
    if (t == "char" || t == "uchar" || t == "int8" || t == "uint8") return 1;
    if (t == "short" || t == "ushort" || t == "int16" || t == "uint16") return 2;
    if (t == "int" || t == "uint" || t == "float" || t == "int32" || t == "uint32" || t == "float32") return 4;
    if (t == "double" || t == "float64") return 8;
    return 0;
}

double read_binary(const unsigned char* p, const std::string& t, bool swap) {
    unsigned char b[8];
    int n = type_size(t);
    for (int i = 0; i < n; ++i) b[i] = swap ? p[n - 1 - i] : p[i];
    if (t == "char" || t == "int8") return (double)(int8_t)b[0];
    if (t == "uchar" || t == "uint8") return (double)b[0];
    if (t == "short" || t == "int16") { int16_t v; memcpy(&v, b, 2); return v; }
    if (t == "ushort" || t == "uint16") { uint16_t v; memcpy(&v, b, 2); return v; }
    if (t == "int" || t == "int32") { int32_t v; memcpy(&v, b, 4); return v; }
    if (t == "uint" || t == "uint32") { uint32_t v; memcpy(&v, b, 4); return v; }
    if (t == "float" || t == "float32") { float v; memcpy(&v, b, 4); return v; }
    double v;
    memcpy(&v, b, 8);
    return v;
}

bool host_little_endian() {
    uint16_t v = 1;
    unsigned char c;
    memcpy(&c, &v, 1);
    return c == 1;
}

struct Prop {
    std::string name, type, count_type;
    bool list = false;
};
struct Elem {
    std::string name;
    long long count = 0;
    std::vector<Prop> props;
};

int read_ply(const char* path) {
    FILE* f = fopen(path, "rb");
    if (!f) { prgpu::set_last_error("cannot open %s", path); return PRGPU_ERR_IO; }
    std::vector<unsigned char> data;
    {
        fseek(f, 0, SEEK_END);
        long sz = ftell(f);
        fseek(f, 0, SEEK_SET);
        data.resize(sz > 0 ? (size_t)sz : 0);
        if (sz > 0 && fread(data.data(), 1, (size_t)sz, f) != (size_t)sz) { fclose(f); return PRGPU_ERR_IO; }
        fclose(f);
    }
    size_t pos = 0;
    auto getline = [&](std::string& line) -> bool {
        if (pos >= data.size()) return false;
        size_t e = pos;
        while (e < data.size() && data[e] != '\n') ++e;
        line.assign((const char*)data.data() + pos, e - pos);
        if (!line.empty() && line.back() == '\r') line.pop_back();
        pos = e + 1;
        return true;
    };
    std::string line;
    if (!getline(line) || line != "ply") { prgpu::set_last_error("%s: not a PLY file", path); return PRGPU_ERR_IO; }
    int fmt = -1;   // 0 ascii, 1 binary le, 2 binary be
    std::vector<Elem> elems;
    while (getline(line)) {
        char w0[64] = {0}, w1[64] = {0}, w2[64] = {0}, w3[64] = {0}, w4[64] = {0};
        int nw = sscanf(line.c_str(), "%63s %63s %63s %63s %63s", w0, w1, w2, w3, w4);
        if (nw <= 0) continue;
        std::string k = w0;
        if (k == "format") {
            std::string t = w1;
            fmt = (t == "ascii") ? 0 : (t == "binary_little_endian") ? 1 : (t == "binary_big_endian") ? 2 : -1;
        } else if (k == "element") {
            Elem e;
            e.name = w1;
            e.count = atoll(w2);
            elems.push_back(e);
        } else if (k == "property" && !elems.empty()) {
            Prop p;
            if (std::string(w1) == "list") { p.list = true; p.count_type = w2; p.type = w3; p.name = w4; }
            else { p.type = w1; p.name = w2; }
            elems.back().props.push_back(p);
        } else if (k == "end_header") {
            break;
        }
    }
    if (fmt < 0) { prgpu::set_last_error("%s: unsupported PLY format", path); return PRGPU_ERR_IO; }
    g_xyz.clear();
    g_nrm.clear();
    const bool swap = (fmt == 1) != host_little_endian();
    const char* want[6] = {"x", "y", "z", "nx", "ny", "nz"};
    for (auto& e : elems) {
        int col[6] = {-1, -1, -1, -1, -1, -1};
        for (size_t i = 0; i < e.props.size(); ++i)
            for (int w = 0; w < 6; ++w)
                if (e.props[i].name == want[w] && !e.props[i].list) col[w] = (int)i;
        const bool is_vertex = e.name == "vertex";
        if (is_vertex) {
            for (int w = 0; w < 6; ++w)
                if (col[w] < 0) { prgpu::set_last_error("%s: vertex lacks %s", path, want[w]); return PRGPU_ERR_IO; }
            g_xyz.resize(3 * e.count);
            g_nrm.resize(3 * e.count);
        }
        for (long long r = 0; r < e.count; ++r) {
            double v[64];
            for (size_t i = 0; i < e.props.size(); ++i) {
                const Prop& p = e.props[i];
                if (fmt == 0) {
                    while (pos < data.size() && isspace(data[pos])) ++pos;
                    if (pos >= data.size()) { prgpu::set_last_error("%s: truncated", path); return PRGPU_ERR_IO; }
                    char* end = nullptr;
                    double x = strtod((const char*)data.data() + pos, &end);
                    if (end == (const char*)data.data() + pos) { prgpu::set_last_error("%s: bad number", path); return PRGPU_ERR_IO; }
                    pos = end - (const char*)data.data();
                    if (p.list) {
                        for (long long q = 0; q < (long long)x; ++q) {
                            while (pos < data.size() && isspace(data[pos])) ++pos;
                            strtod((const char*)data.data() + pos, &end);
                            pos = end - (const char*)data.data();
                        }
                    } else if (i < 64) v[i] = x;
                } else {
                    if (p.list) {
                        int cs = type_size(p.count_type), es = type_size(p.type);
                        if (!cs || !es || pos + cs > data.size()) { prgpu::set_last_error("%s: truncated", path); return PRGPU_ERR_IO; }
                        long long cnt = (long long)read_binary(&data[pos], p.count_type, swap);
                        pos += cs + (size_t)(cnt * es);
                    } else {
                        int ts = type_size(p.type);
                        if (!ts || pos + ts > data.size()) { prgpu::set_last_error("%s: truncated", path); return PRGPU_ERR_IO; }
                        if (i < 64) v[i] = read_binary(&data[pos], p.type, swap);
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
        FILE* f = fopen(path, "rb");
        if (!f) { prgpu::set_last_error("cannot open %s", path); return PRGPU_ERR_IO; }
        g_xyz.clear();
        g_nrm.clear();
        std::string e6 = p.size() >= 6 ? p.substr(p.size() - 6) : "";
        if (e6 == ".bnpts") {
            float b[6];
            while (fread(b, sizeof(float), 6, f) == 6)
                for (int w = 0; w < 3; ++w) { g_xyz.push_back(b[w]); g_nrm.push_back(b[3 + w]); }
        } else {
            float b[6];
            while (fscanf(f, " %f %f %f %f %f %f ", &b[0], &b[1], &b[2], &b[3], &b[4], &b[5]) == 6)
                for (int w = 0; w < 3; ++w) { g_xyz.push_back(b[w]); g_nrm.push_back(b[3 + w]); }
        }
        fclose(f);
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
    FILE* f = fopen(path, "wb");
    if (!f) { prgpu::set_last_error("cannot write %s", path); return PRGPU_ERR_IO; }
    fprintf(f, "ply\nformat %s 1.0\nelement vertex %lld\nproperty float x\nproperty float y\nproperty float z\n"
               "element face %lld\nproperty list uchar int vertex_indices\nend_header\n",
            binary ? "binary_little_endian" : "ascii", (long long)m->n_vertices, (long long)m->n_triangles);
    if (binary) {
        if (!host_little_endian()) { fclose(f); prgpu::set_last_error("big-endian host"); return PRGPU_ERR_IO; }
        fwrite(m->vertices, sizeof(float), (size_t)(3 * m->n_vertices), f);
        std::vector<unsigned char> buf;
        buf.resize((size_t)m->n_triangles * 13);
        for (int64_t t = 0; t < m->n_triangles; ++t) {
            buf[13 * t] = 3;
            memcpy(&buf[13 * t + 1], &m->triangles[3 * t], 12);
        }
        fwrite(buf.data(), 1, buf.size(), f);
    } else {
        for (int64_t v = 0; v < m->n_vertices; ++v)
            fprintf(f, "%g %g %g\n", m->vertices[3 * v], m->vertices[3 * v + 1], m->vertices[3 * v + 2]);
        for (int64_t t = 0; t < m->n_triangles; ++t)
            fprintf(f, "3 %d %d %d\n", m->triangles[3 * t], m->triangles[3 * t + 1], m->triangles[3 * t + 2]);
    }
    int bad = ferror(f);
    fclose(f);
    return bad ? PRGPU_ERR_IO : PRGPU_OK;
}

}  // extern "C"
