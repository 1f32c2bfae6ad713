// Synthetic scene generators and Wavefront OBJ I/O (host C++, no CUDA).
//
// The reference ships no scene assets, so every workload is generated here from a seed:
//   * procedural asteroid: icosphere (recursive midpoint subdivision on the unit sphere),
//     seeded random edge collapse down to a target triangle count, then radial displacement
//     by multi-octave value noise;
//   * vertex normals computed the way the reference OBJ loader computes them
//     (lib/model_loaders/obj.hpp:86-114: sum of the left-handed face normals
//     cross(p0-p1, p2-p0) of every incident face, then normalised);
//   * an OBJ reader that follows obj::load_from_stream (obj.hpp:59-117): `v` lines parsed
//     with strtof, `f` lines fan-triangulated, negative indices allowed, `vt`/`vn` ignored.
//
// Only +,-,*,/ and sqrt are used on floating-point values (all correctly rounded) and the
// library is compiled with -ffp-contract=off, so x86-64 and aarch64 hosts generate
// bit-identical meshes from the same seed.
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <cmath>
#include <vector>
#include <array>
#include <algorithm>
#include <string>
#include <fstream>

namespace {

struct V3 { double x, y, z; };
inline V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 operator*(V3 a, double s) { return {a.x * s, a.y * s, a.z * s}; }
inline double dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 cross(V3 a, V3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
inline V3 normalize(V3 a) { double l = std::sqrt(dot(a, a)); return a * (1.0 / l); }

inline uint64_t splitmix64(uint64_t& s) {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// ---------------------------------------------------------------- icosphere
struct EdgeMap {  // open addressing, key = (min << 32) | max, value = midpoint vertex index
    std::vector<uint64_t> keys;
    std::vector<int32_t> vals;
    uint64_t mask;
    explicit EdgeMap(size_t expected) {
        size_t cap = 1;
        while (cap < expected * 2) cap <<= 1;
        keys.assign(cap, ~0ull);
        vals.assign(cap, -1);
        mask = cap - 1;
    }
    int32_t* find_or_insert(uint64_t key, bool& inserted) {
        uint64_t h = key * 0x9E3779B97F4A7C15ull;
        size_t i = (size_t)(h >> 17) & mask;
        while (true) {
            if (keys[i] == key) { inserted = false; return &vals[i]; }
            if (keys[i] == ~0ull) { keys[i] = key; inserted = true; return &vals[i]; }
            i = (i + 1) & mask;
        }
    }
};

void icosphere(int level, std::vector<V3>& P, std::vector<std::array<int32_t, 3>>& F) {
    const double t = (1.0 + std::sqrt(5.0)) / 2.0;
    const V3 base[12] = {{-1, t, 0}, {1, t, 0}, {-1, -t, 0}, {1, -t, 0}, {0, -1, t}, {0, 1, t},
                         {0, -1, -t}, {0, 1, -t}, {t, 0, -1}, {t, 0, 1}, {-t, 0, -1}, {-t, 0, 1}};
    // Counter-clockwise seen from outside: outward right-handed normals.
    const int faces[20][3] = {{0, 11, 5}, {0, 5, 1}, {0, 1, 7}, {0, 7, 10}, {0, 10, 11},
                              {1, 5, 9}, {5, 11, 4}, {11, 10, 2}, {10, 7, 6}, {7, 1, 8},
                              {3, 9, 4}, {3, 4, 2}, {3, 2, 6}, {3, 6, 8}, {3, 8, 9},
                              {4, 9, 5}, {2, 4, 11}, {6, 2, 10}, {8, 6, 7}, {9, 8, 1}};
    P.clear();
    F.clear();
    for (auto& b : base) P.push_back(normalize(b));
    for (auto& f : faces) F.push_back({f[0], f[1], f[2]});
    for (int l = 0; l < level; ++l) {
        EdgeMap em(F.size() * 3 / 2 + 16);
        std::vector<std::array<int32_t, 3>> NF;
        NF.reserve(F.size() * 4);
        P.reserve(P.size() + F.size() * 3 / 2 + 16);
        auto mid = [&](int32_t a, int32_t b) -> int32_t {
            uint64_t key = a < b ? ((uint64_t)a << 32) | (uint32_t)b : ((uint64_t)b << 32) | (uint32_t)a;
            bool ins;
            int32_t* v = em.find_or_insert(key, ins);
            if (ins) {
                *v = (int32_t)P.size();
                P.push_back(normalize((P[a] + P[b]) * 0.5));
            }
            return *v;
        };
        for (auto& f : F) {
            int32_t a = mid(f[0], f[1]), b = mid(f[1], f[2]), c = mid(f[2], f[0]);
            NF.push_back({f[0], a, c});
            NF.push_back({f[1], b, a});
            NF.push_back({f[2], c, b});
            NF.push_back({a, b, c});
        }
        F.swap(NF);
    }
}

// ---------------------------------------------------------------- decimation
// Seeded random half-edge collapse on a closed 2-manifold lying on the unit sphere.
// Each pass shuffles the live edges and collapses every edge whose endpoints are still
// untouched in that pass, subject to: the edge is manifold (exactly two incident faces),
// the link condition holds (the endpoints share exactly the two opposite vertices),
// the merged vertex valence stays <= 12, and no surviving face flips or becomes a sliver
// once the merged vertex moves to the normalised midpoint. Every collapse removes two faces.
struct Decimator {
    std::vector<V3>& P;
    std::vector<std::array<int32_t, 3>>& F;
    std::vector<uint8_t> dead;
    std::vector<int32_t> parent;
    std::vector<std::vector<int32_t>> vf;
    size_t alive;

    Decimator(std::vector<V3>& p, std::vector<std::array<int32_t, 3>>& f) : P(p), F(f) {
        dead.assign(F.size(), 0);
        parent.resize(P.size());
        for (size_t i = 0; i < P.size(); ++i) parent[i] = (int32_t)i;
        vf.resize(P.size());
        for (size_t i = 0; i < F.size(); ++i)
            for (int k = 0; k < 3; ++k) vf[F[i][k]].push_back((int32_t)i);
        alive = F.size();
    }
    int32_t find(int32_t v) {
        while (parent[v] != v) { parent[v] = parent[parent[v]]; v = parent[v]; }
        return v;
    }
    void corners(int32_t f, int32_t c[3]) { for (int k = 0; k < 3; ++k) c[k] = find(F[f][k]); }
    void neighbours(int32_t v, std::vector<int32_t>& out) {
        out.clear();
        for (int32_t f : vf[v]) {
            if (dead[f]) continue;
            int32_t c[3];
            corners(f, c);
            for (int k = 0; k < 3; ++k)
                if (c[k] != v) out.push_back(c[k]);
        }
        std::sort(out.begin(), out.end());
        out.erase(std::unique(out.begin(), out.end()), out.end());
    }
    bool try_collapse(int32_t a, int32_t b, std::vector<int32_t>& na, std::vector<int32_t>& nb) {
        // faces shared by a and b
        int32_t shared[2];
        int ns = 0;
        for (int32_t f : vf[a]) {
            if (dead[f]) continue;
            int32_t c[3];
            corners(f, c);
            if (c[0] == b || c[1] == b || c[2] == b) {
                if (ns == 2) return false;
                shared[ns++] = f;
            }
        }
        if (ns != 2) return false;
        neighbours(a, na);
        neighbours(b, nb);
        size_t common = 0;
        for (size_t i = 0, j = 0; i < na.size() && j < nb.size();) {
            if (na[i] < nb[j]) ++i;
            else if (na[i] > nb[j]) ++j;
            else { ++common; ++i; ++j; }
        }
        if (common != 2) return false;
        if (na.size() + nb.size() - 4 > 12) return false;
        V3 m = normalize(P[a] + P[b]);
        // fold-over / sliver check on every face that survives around a or b
        for (int side = 0; side < 2; ++side) {
            int32_t v = side ? b : a;
            for (int32_t f : vf[v]) {
                if (dead[f] || f == shared[0] || f == shared[1]) continue;
                int32_t c[3];
                corners(f, c);
                V3 q[3];
                for (int k = 0; k < 3; ++k) q[k] = (c[k] == a || c[k] == b) ? m : P[c[k]];
                V3 n = cross(q[1] - q[0], q[2] - q[0]);
                double nl2 = dot(n, n);
                V3 cen = (q[0] + q[1] + q[2]) * (1.0 / 3.0);
                double d = dot(n, cen);
                if (!(d > 0.0)) return false;
                // cosine between face normal and radial direction must stay above 0.5
                if (d * d < 0.25 * nl2 * dot(cen, cen)) return false;
                // aspect guard: squared area vs squared longest edge
                double e0 = dot(q[1] - q[0], q[1] - q[0]), e1 = dot(q[2] - q[1], q[2] - q[1]),
                       e2 = dot(q[0] - q[2], q[0] - q[2]);
                double emax = std::max(e0, std::max(e1, e2));
                if (nl2 < 0.02 * emax * emax) return false;
            }
        }
        dead[shared[0]] = dead[shared[1]] = 1;
        alive -= 2;
        parent[b] = a;
        P[a] = m;
        std::vector<int32_t> merged;
        merged.reserve(vf[a].size() + vf[b].size());
        for (int32_t f : vf[a]) if (!dead[f]) merged.push_back(f);
        for (int32_t f : vf[b]) if (!dead[f]) merged.push_back(f);
        vf[a].swap(merged);
        std::vector<int32_t>().swap(vf[b]);
        return true;
    }
    bool run(size_t target, uint64_t seed) {
        uint64_t rng = seed * 0xD1B54A32D192ED03ull + 0x2545F4914F6CDD1Dull;
        std::vector<uint8_t> touched(P.size());
        std::vector<uint64_t> edges;
        std::vector<int32_t> na, nb;
        for (int pass = 0; pass < 200 && alive > target; ++pass) {
            edges.clear();
            for (size_t f = 0; f < F.size(); ++f) {
                if (dead[f]) continue;
                int32_t c[3];
                corners((int32_t)f, c);
                for (int k = 0; k < 3; ++k) {
                    int32_t a = c[k], b = c[(k + 1) % 3];
                    if (a < b) edges.push_back(((uint64_t)a << 32) | (uint32_t)b);
                }
            }
            for (size_t i = edges.size(); i > 1; --i) {
                size_t j = (size_t)(splitmix64(rng) % i);
                std::swap(edges[i - 1], edges[j]);
            }
            std::fill(touched.begin(), touched.end(), 0);
            size_t done = 0;
            for (uint64_t e : edges) {
                if (alive <= target) break;
                int32_t a = find((int32_t)(e >> 32)), b = find((int32_t)(e & 0xffffffffu));
                if (a == b || touched[a] || touched[b]) continue;
                if (try_collapse(a, b, na, nb)) { touched[a] = touched[b] = 1; ++done; }
            }
            if (done == 0) break;
        }
        return alive == target;
    }
    void compact() {
        std::vector<int32_t> remap(P.size(), -1);
        std::vector<V3> NP;
        std::vector<std::array<int32_t, 3>> NF;
        NF.reserve(alive);
        for (size_t f = 0; f < F.size(); ++f) {
            if (dead[f]) continue;
            int32_t c[3];
            corners((int32_t)f, c);
            std::array<int32_t, 3> nf;
            for (int k = 0; k < 3; ++k) {
                if (remap[c[k]] < 0) { remap[c[k]] = (int32_t)NP.size(); NP.push_back(P[c[k]]); }
                nf[k] = remap[c[k]];
            }
            NF.push_back(nf);
        }
        P.swap(NP);
        F.swap(NF);
    }
};

// ---------------------------------------------------------------- value noise
inline uint32_t hash4(int32_t x, int32_t y, int32_t z, uint32_t seed) {
    uint32_t h = seed * 0x27d4eb2du;
    h ^= (uint32_t)x * 0x85ebca6bu; h = (h << 13) | (h >> 19); h *= 0xc2b2ae35u;
    h ^= (uint32_t)y * 0x9e3779b1u; h = (h << 17) | (h >> 15); h *= 0x85ebca6bu;
    h ^= (uint32_t)z * 0xc2b2ae3du; h = (h << 11) | (h >> 21); h *= 0x27d4eb2fu;
    h ^= h >> 16; h *= 0x7feb352du; h ^= h >> 15; h *= 0x846ca68bu; h ^= h >> 16;
    return h;
}
inline double lattice(int32_t x, int32_t y, int32_t z, uint32_t seed) {
    return (double)(hash4(x, y, z, seed) >> 8) * (2.0 / 16777215.0) - 1.0;  // [-1, 1]
}
inline double fade(double t) { return t * t * t * (t * (t * 6.0 - 15.0) + 10.0); }
double value_noise(V3 p, uint32_t seed) {
    double fx = std::floor(p.x), fy = std::floor(p.y), fz = std::floor(p.z);
    int32_t ix = (int32_t)fx, iy = (int32_t)fy, iz = (int32_t)fz;
    double tx = fade(p.x - fx), ty = fade(p.y - fy), tz = fade(p.z - fz);
    double c[2][2][2];
    for (int a = 0; a < 2; ++a)
        for (int b = 0; b < 2; ++b)
            for (int d = 0; d < 2; ++d) c[a][b][d] = lattice(ix + a, iy + b, iz + d, seed);
    auto lerp = [](double a, double b, double t) { return a + (b - a) * t; };
    double x00 = lerp(c[0][0][0], c[1][0][0], tx), x10 = lerp(c[0][1][0], c[1][1][0], tx);
    double x01 = lerp(c[0][0][1], c[1][0][1], tx), x11 = lerp(c[0][1][1], c[1][1][1], tx);
    return lerp(lerp(x00, x10, ty), lerp(x01, x11, ty), tz);
}
double fbm(V3 p, int octaves, double base_freq, uint32_t seed) {
    double sum = 0.0, norm = 0.0, amp = 1.0, freq = base_freq;
    for (int o = 0; o < octaves; ++o) {
        // per-octave offset decorrelates the lattices of successive octaves
        V3 q = {p.x * freq + 17.25 * o, p.y * freq - 31.5 * o, p.z * freq + 7.125 * o};
        sum += amp * value_noise(q, seed + 0x9E37u * (uint32_t)o);
        norm += amp;
        amp *= 0.5;
        freq *= 2.0;
    }
    return sum / norm;
}

}  // namespace

extern "C" {

// Vertex normals as the reference OBJ loader computes them (obj.hpp:86-114): every face adds
// its left-handed normal cross(p0-p1, p2-p0) (un-normalised, i.e. area weighted) to its three
// vertices; the sums are then normalised. Inputs are float32 positions widened to double, as
// the reference stores them. Output: n_vertices x 3 doubles.
void crt_mesh_vertex_normals(const float* xyz, size_t n_vertices, const int32_t* faces, size_t n_faces,
                             double* out_normals) {
    std::fill(out_normals, out_normals + 3 * n_vertices, 0.0);
    for (size_t f = 0; f < n_faces; ++f) {
        const int32_t* c = faces + 3 * f;
        V3 p0 = {xyz[3 * c[0]], xyz[3 * c[0] + 1], xyz[3 * c[0] + 2]};
        V3 p1 = {xyz[3 * c[1]], xyz[3 * c[1] + 1], xyz[3 * c[1] + 2]};
        V3 p2 = {xyz[3 * c[2]], xyz[3 * c[2] + 1], xyz[3 * c[2] + 2]};
        V3 n = cross(p0 - p1, p2 - p0);
        for (int k = 0; k < 3; ++k) {
            out_normals[3 * c[k]] += n.x;
            out_normals[3 * c[k] + 1] += n.y;
            out_normals[3 * c[k] + 2] += n.z;
        }
    }
    for (size_t v = 0; v < n_vertices; ++v) {
        V3 n = {out_normals[3 * v], out_normals[3 * v + 1], out_normals[3 * v + 2]};
        double inv = 1.0 / std::sqrt(dot(n, n));
        out_normals[3 * v] = n.x * inv;
        out_normals[3 * v + 1] = n.y * inv;
        out_normals[3 * v + 2] = n.z * inv;
    }
}

// Procedural asteroid. Returns 0 on success, writes counts to *n_vertices / *n_faces and, when
// the output pointers are non-NULL and the capacities suffice, the float32 vertices and int32 faces.
// Call once with NULL outputs to learn the sizes (the mesh is regenerated on each call).
//   level          icosphere subdivision level (20 * 4^level faces before decimation)
//   target_faces   faces after random edge collapse (even, <= 20*4^level; 0 = no decimation)
//   radius         mean radius in metres
//   amplitude      relative radial displacement amplitude (0.05 = 5 %)
//   octaves        value-noise octaves
//   seed           seeds both the collapse order and the noise lattice
int crt_scene_asteroid(int level, size_t target_faces, double radius, double amplitude, int octaves,
                       uint64_t seed, float* out_xyz, size_t cap_vertices, int32_t* out_faces,
                       size_t cap_faces, size_t* n_vertices, size_t* n_faces) {
    if (level < 0 || level > 11 || octaves < 1 || octaves > 16) return -1;
    std::vector<V3> P;
    std::vector<std::array<int32_t, 3>> F;
    icosphere(level, P, F);
    if (target_faces && target_faces < F.size()) {
        if (target_faces % 2 || target_faces < 20) return -1;
        Decimator d(P, F);
        if (!d.run(target_faces, seed)) return -2;
        d.compact();
    }
    *n_vertices = P.size();
    *n_faces = F.size();
    if (!out_xyz || !out_faces) return 0;
    if (cap_vertices < P.size() || cap_faces < F.size()) return -3;
    const uint32_t nseed = (uint32_t)(seed ^ (seed >> 32)) * 2654435761u + 12345u;
    for (size_t i = 0; i < P.size(); ++i) {
        V3 u = P[i];
        double r = radius * (1.0 + amplitude * fbm(u, octaves, 1.5, nseed));
        out_xyz[3 * i] = (float)(u.x * r);
        out_xyz[3 * i + 1] = (float)(u.y * r);
        out_xyz[3 * i + 2] = (float)(u.z * r);
    }
    std::memcpy(out_faces, F.data(), F.size() * sizeof(F[0]));
    return 0;
}

// Writes an indexed mesh as Wavefront OBJ ('%.9g' round-trips float32 exactly). Returns 0 on success.
int crt_obj_write(const char* path, const float* xyz, size_t n_vertices, const int32_t* faces, size_t n_faces) {
    FILE* f = std::fopen(path, "w");
    if (!f) return -1;
    std::vector<char> buf(1 << 20);
    std::setvbuf(f, buf.data(), _IOFBF, buf.size());
    for (size_t v = 0; v < n_vertices; ++v)
        std::fprintf(f, "v %.9g %.9g %.9g\n", xyz[3 * v], xyz[3 * v + 1], xyz[3 * v + 2]);
    for (size_t t = 0; t < n_faces; ++t)
        std::fprintf(f, "f %d %d %d\n", faces[3 * t] + 1, faces[3 * t + 1] + 1, faces[3 * t + 2] + 1);
    int rc = std::ferror(f) ? -2 : 0;
    std::fclose(f);
    return rc;
}

}  // extern "C"
