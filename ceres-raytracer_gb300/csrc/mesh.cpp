// Wavefront OBJ ingest for entities (host C++).
//
// Follows obj::load_from_stream (lib/model_loaders/obj.hpp:59-117): lines are read up to 1024
// characters, `v x y z` parsed with strtof, `f` lines fan-triangulated from their first vertex,
// indices may be negative (relative to the vertices read so far) and may carry /vt/vn parts, which
// are ignored; per-vertex normals are the normalised sums of the left-handed face normals
// cross(p0 - p1, p2 - p0) of all incident faces, computed in FP64.
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "crt_gpu.h"

struct crt_mesh {
    std::vector<float> xyz;      // 9 per triangle
    std::vector<float> normals;  // 9 per triangle
};

namespace {

char* strip_spaces(char* p) {
    while (std::isspace((unsigned char)*p)) ++p;
    return p;
}

void remove_eol(char* p) {
    long i = (long)std::strlen(p) - 1;
    while (i > 0 && std::isspace((unsigned char)p[i])) p[i--] = '\0';
}

struct FileCloser {
    void operator()(FILE* f) const { std::fclose(f); }
};

// obj.hpp:31-55 read_index
bool read_index(char** ptr, long* out) {
    char* base = strip_spaces(*ptr);
    if (!std::isdigit((unsigned char)*base) && *base != '-') return false;
    long index = std::strtol(base, &base, 10);
    base = strip_spaces(base);
    if (*base == '/') {
        ++base;
        if (*base != '/') std::strtol(base, &base, 10);
        base = strip_spaces(base);
        if (*base == '/') {
            ++base;
            std::strtol(base, &base, 10);
        }
    }
    *ptr = base;
    *out = index;
    return true;
}

}  // namespace

extern "C" {

int crt_mesh_load_obj(const char* path, crt_mesh** out) {
    if (!path || !out) return CRT_ERR_INVALID;
    *out = nullptr;
    // the file is closed on every return, also when an allocation fails mid-parse
    std::unique_ptr<FILE, FileCloser> file(std::fopen(path, "r"));
    FILE* f = file.get();
    if (!f) return CRT_ERR_IO;
    crt_mesh* m = new (std::nothrow) crt_mesh();
    if (!m) return CRT_ERR_OOM;
    std::vector<float> vx;                  // vertices, 3 per vertex (float32 as parsed)
    std::vector<double> acc;                // accumulated normals, 3 per vertex
    std::vector<long> tri_idx;              // 3 per triangle
    char line[1024];
    try {
        while (std::fgets(line, sizeof(line), f)) {
            // over-long line: its first 1023 characters are parsed and the rest is skipped.  (The
            // reference's istream::getline sets failbit there and its loop ends, silently dropping
            // the rest of the file; this loader reads on.)
            size_t len = std::strlen(line);
            if (len == sizeof(line) - 1 && line[len - 1] != '\n') {
                int c;
                while ((c = std::fgetc(f)) != EOF && c != '\n') {
                }
            }
            char* p = strip_spaces(line);
            if (*p == '\0' || *p == '#') continue;
            remove_eol(p);
            if (p[0] == 'v' && std::isspace((unsigned char)p[1])) {
                char* q = p + 1;
                float x = std::strtof(q, &q);
                float y = std::strtof(q, &q);
                float z = std::strtof(q, &q);
                vx.push_back(x);
                vx.push_back(y);
                vx.push_back(z);
                acc.push_back(0.0);
                acc.push_back(0.0);
                acc.push_back(0.0);
            } else if (p[0] == 'f' && std::isspace((unsigned char)p[1])) {
                char* q = p + 2;
                long idx[2] = {0, 0};
                long index;
                for (size_t i = 0; read_index(&q, &index); ++i) {
                    const long nv = (long)(vx.size() / 3);
                    long j = index < 0 ? nv + index : index - 1;
                    if (j < 0 || j >= nv) {   // index 0, past the last vertex, or before the first
                        delete m;
                        return CRT_ERR_IO;
                    }
                    if (i >= 2) {
                        const long t[3] = {idx[0], idx[1], j};
                        for (int k = 0; k < 3; ++k) tri_idx.push_back(t[k]);
                        // left-handed face normal cross(p0 - p1, p2 - p0) in FP64
                        double P[3][3];
                        for (int k = 0; k < 3; ++k)
                            for (int c = 0; c < 3; ++c) P[k][c] = vx[3 * t[k] + c];
                        const double e1[3] = {P[0][0] - P[1][0], P[0][1] - P[1][1], P[0][2] - P[1][2]};
                        const double e2[3] = {P[2][0] - P[0][0], P[2][1] - P[0][1], P[2][2] - P[0][2]};
                        const double n[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2],
                                             e1[0] * e2[1] - e1[1] * e2[0]};
                        for (int k = 0; k < 3; ++k)
                            for (int c = 0; c < 3; ++c) acc[3 * t[k] + c] += n[c];
                        idx[1] = j;
                    } else {
                        idx[i] = j;
                    }
                }
            }
        }
        file.reset();
        const size_t nt = tri_idx.size() / 3;
        m->xyz.resize(nt * 9);
        m->normals.resize(nt * 9);
        for (size_t v = 0; v < acc.size() / 3; ++v) {
            const double l = std::sqrt(acc[3 * v] * acc[3 * v] + acc[3 * v + 1] * acc[3 * v + 1] +
                                       acc[3 * v + 2] * acc[3 * v + 2]);
            const double inv = 1.0 / l;
            for (int c = 0; c < 3; ++c) acc[3 * v + c] *= inv;
        }
        for (size_t t = 0; t < nt; ++t)
            for (int k = 0; k < 3; ++k)
                for (int c = 0; c < 3; ++c) {
                    m->xyz[9 * t + 3 * k + c] = vx[3 * tri_idx[3 * t + k] + c];
                    m->normals[9 * t + 3 * k + c] = (float)acc[3 * tri_idx[3 * t + k] + c];
                }
    } catch (const std::bad_alloc&) {
        delete m;
        return CRT_ERR_OOM;
    }
    *out = m;
    return CRT_OK;
}

size_t crt_mesh_num_tris(const crt_mesh* m) { return m ? m->xyz.size() / 9 : 0; }
const float* crt_mesh_xyz(const crt_mesh* m) { return m ? m->xyz.data() : nullptr; }
const float* crt_mesh_normals(const crt_mesh* m) { return m ? m->normals.data() : nullptr; }
void crt_mesh_destroy(crt_mesh* m) { delete m; }

}  // extern "C"
