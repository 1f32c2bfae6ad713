// `_crt` extension module: the pybind11 surface of the reference module (src/pybind.cpp:130-719)
// over the C ABI of libcrt_gpu.so.
//
// Same class names, constructors, methods, positional arguments and return shapes/dtypes as the
// reference: SimpleCamera, SimpleLidar, PointLight, AreaLight, Entity, BodyFixedEntity,
// BodyFixedGroup and the free functions render / simulate_lidar / intersection_pass /
// instance_pass / normal_pass.  Extensions are keyword arguments or new methods only:
//   render(..., seed=0, request=0, return_radiance=False)
//   SimpleLidar.set_beam_grid(nx, ny, half_angle_x, half_angle_y) + BodyFixedGroup.lidar_scan(lidar)
//   BodyFixedEntity/Entity.set_reflectivity(specular, diffuse) + BodyFixedGroup.srp(...)
//   set_device(i), synchronize(), scene_stats on BodyFixedGroup.
// Device work runs with the GIL released; one module-wide mutex serialises use of the context.
#include <pybind11/numpy.h>
#include <pybind11/pybind11.h>
#include <pybind11/stl.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <map>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

#include "crt_gpu.h"

namespace py = pybind11;
using f64arr = py::array_t<double, py::array::c_style | py::array::forcecast>;

namespace {

std::mutex g_mu;
crt_context* g_ctx = nullptr;
int g_device = 0;

[[noreturn]] void raise_status(int rc, const std::string& where) {
    std::string msg = where + ": " + crt_status_string(rc);
    if (g_ctx) msg += " (" + std::string(crt_context_last_error(g_ctx)) + ")";
    if (rc == CRT_ERR_OOM) throw std::bad_alloc();
    if (rc == CRT_ERR_INVALID) throw py::value_error(msg);
    throw std::runtime_error(msg);
}

crt_context* ctx() {
    if (!g_ctx) {
        const char* env = std::getenv("CRT_DEVICE");
        int dev = env ? std::atoi(env) : g_device;
        int rc = crt_context_create(dev, &g_ctx);
        if (rc != CRT_OK) {
            g_ctx = nullptr;
            throw std::runtime_error(std::string("_crt: cannot create a GPU context: ") + crt_status_string(rc) +
                                     " (the ray-query path runs on the GPU only)");
        }
    }
    return g_ctx;
}

// Page-locked result arrays: renders, passes and scans return numpy arrays whose memory comes from
// crt_host_alloc, so the device-to-host copies run at the full host link rate.  Buffers of released
// arrays are kept for reuse, up to 1 GiB.  The pool is never destroyed (arrays may outlive the
// module's static objects at interpreter exit).
struct PinnedPool {
    std::mutex mu;
    std::multimap<size_t, void*> free_;
    size_t cached = 0;
    void* get(size_t n, size_t& cap) {
        {
            std::lock_guard<std::mutex> lk(mu);
            auto it = free_.lower_bound(n);
            if (it != free_.end() && it->first <= 2 * n + 4096) {
                cap = it->first;
                void* p = it->second;
                cached -= cap;
                free_.erase(it);
                return p;
            }
        }
        void* p = nullptr;
        if (crt_host_alloc(n, &p) != CRT_OK || !p) throw std::bad_alloc();
        cap = n;
        return p;
    }
    void put(void* p, size_t cap) {
        std::lock_guard<std::mutex> lk(mu);
        if (cached + cap > ((size_t)1 << 30)) {
            crt_host_free(p);
            return;
        }
        free_.emplace(cap, p);
        cached += cap;
    }
};

PinnedPool& pinned_pool() {
    static PinnedPool* pool = new PinnedPool();
    return *pool;
}

struct PinnedBlock {
    void* p;
    size_t cap;
};

template <class T>
py::array_t<T> pinned_array(std::vector<py::ssize_t> shape) {
    size_t n = sizeof(T);
    for (py::ssize_t d : shape) n *= (size_t)d;
    size_t cap = 0;
    void* p = pinned_pool().get(std::max<size_t>(n, 1), cap);
    auto* blk = new PinnedBlock{p, cap};
    py::capsule owner(blk, [](void* q) {
        PinnedBlock* b = static_cast<PinnedBlock*>(q);
        pinned_pool().put(b->p, b->cap);
        delete b;
    });
    return py::array_t<T>(shape, static_cast<T*>(p), owner);
}

bool verbose() {
    const char* v = std::getenv("CRT_VERBOSE");
    return v && v[0] == '1';
}

void read3(const py::handle& h, double out[3]) {
    f64arr a = py::cast<f64arr>(h);
    if (a.size() < 3) throw py::value_error("expected 3 values");
    const double* p = a.data();
    for (int k = 0; k < 3; ++k) out[k] = p[k];
}
void read9(const py::handle& h, double out[9]) {
    f64arr a = py::cast<f64arr>(h);
    if (a.size() < 9) throw py::value_error("expected a 3x3 rotation");
    const double* p = a.data();
    for (int k = 0; k < 9; ++k) out[k] = p[k];
}

// RigidBody (src/crt/rigid_body.hpp:7-49)
struct Pose {
    double position[3] = {0, 0, 0};
    double rotation[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
    void set_position(const py::handle& p) { read3(p, position); }
    void set_rotation(const py::handle& r) { read9(r, rotation); }
    void set_pose(const py::handle& p, const py::handle& r) {
        read3(p, position);
        read9(r, rotation);
    }
};

struct SimpleCamera : Pose {
    double focal_length;
    double resolution[2];
    double sensor_size[2];
    bool z_positive;
    SimpleCamera(double f, const py::sequence& res, const py::sequence& sensor, bool zpos) {
        focal_length = f;
        resolution[0] = py::cast<double>(res[0]);
        resolution[1] = py::cast<double>(res[1]);
        sensor_size[0] = py::cast<double>(sensor[0]);
        sensor_size[1] = py::cast<double>(sensor[1]);
        z_positive = zpos;
    }
    crt_camera_desc desc() const {
        crt_camera_desc c;
        std::copy(position, position + 3, c.position);
        std::copy(rotation, rotation + 9, c.rotation);
        c.focal_length = focal_length;
        c.resolution[0] = resolution[0];
        c.resolution[1] = resolution[1];
        c.sensor_size[0] = sensor_size[0];
        c.sensor_size[1] = sensor_size[1];
        c.z_positive = z_positive ? 1 : 0;
        return c;
    }
    int width() const { return (int)std::floor(resolution[0]); }
    int height() const { return (int)std::floor(resolution[1]); }
};

struct SimpleLidar : Pose {
    bool z_positive;
    std::vector<double> batch_positions;   // n * 3
    std::vector<double> batch_rotations;   // n * 9 (row-major per pose)
    uint32_t nx = 0, ny = 0;
    double half_x = 0, half_y = 0;
    explicit SimpleLidar(bool zpos) : z_positive(zpos) {}
    // batch_set_pose(positions [n, 3], rotations [3, 3, 100000], n)  (src/pybind.cpp:216-247)
    void batch_set_pose(const f64arr& pos, const f64arr& rot, int n) {
        if (n < 0 || n > 100000) throw py::value_error("number_of_poses must be in [0, 100000]");
        if (pos.size() < 3 * (py::ssize_t)n) throw py::value_error("batch_positions has fewer than n poses");
        if (rot.size() < 9 * 100000) throw py::value_error("batch_rotations must have shape (3, 3, 100000)");
        const double* p = pos.data();
        const double* r = rot.data();
        batch_positions.assign(p, p + 3 * (size_t)n);
        batch_rotations.resize(9 * (size_t)n);
        for (int k = 0; k < n; ++k)
            for (int i = 0; i < 3; ++i)
                for (int j = 0; j < 3; ++j) batch_rotations[9 * (size_t)k + 3 * i + j] = r[(3 * i + j) * 100000 + k];
    }
    void set_beam_grid(uint32_t x, uint32_t y, double hx, double hy) {
        nx = x;
        ny = y;
        half_x = hx;
        half_y = hy;
    }
};

struct PointLight : Pose {
    double intensity;
    explicit PointLight(double i) : intensity(i) {}
};

struct AreaLight : Pose {
    double intensity;
    double size[2];
    AreaLight(double i, const py::sequence& s) : intensity(i) {
        size[0] = py::cast<double>(s[0]);
        size[1] = py::cast<double>(s[1]);
    }
};

// Entity (src/crt/rendering_dynamic/entity.hpp:21-86): mesh loaded once in the constructor
struct Mesh {
    std::vector<float> xyz, vn;
    size_t n = 0;
};

std::shared_ptr<Mesh> load_mesh(const std::string& path, std::string type) {
    std::transform(type.begin(), type.end(), type.begin(), [](unsigned char c) { return (char)std::tolower(c); });
    auto m = std::make_shared<Mesh>();
    if (type != "obj") {
        if (verbose()) std::printf("file type of %s is not a valid.  crt currently supports obj\n", type.c_str());
        return m;   // the reference loads no triangles for other types (entity.hpp:38-41)
    }
    crt_mesh* h = nullptr;
    int rc = crt_mesh_load_obj(path.c_str(), &h);
    if (rc == CRT_ERR_IO) {   // unreadable file: the reference loads an empty mesh (obj.hpp:120-125)
        if (verbose()) std::printf("0 triangles loaded from %s\n", path.c_str());
        return m;
    }
    if (rc != CRT_OK) raise_status(rc, "load_obj");
    m->n = crt_mesh_num_tris(h);
    m->xyz.assign(crt_mesh_xyz(h), crt_mesh_xyz(h) + 9 * m->n);
    m->vn.assign(crt_mesh_normals(h), crt_mesh_normals(h) + 9 * m->n);
    crt_mesh_destroy(h);
    if (verbose()) std::printf("%zu triangles loaded from %s\n", m->n, path.c_str());
    return m;
}

struct EntityBase : Pose {
    std::string geometry_path, geometry_type;
    bool smooth_shading;
    float color[3];
    double scale = 1.0;
    float rho_s = 0.f, rho_d = 0.f;
    uint32_t id = 0;
    EntityBase(const std::string& path, const std::string& type, bool smooth, const py::sequence& c)
        : geometry_path(path), geometry_type(type), smooth_shading(smooth) {
        for (int k = 0; k < 3; ++k) color[k] = py::cast<float>(c[k]);
    }
    void set_scale(double s) { scale = s; }
    void set_reflectivity(double s, double d) {
        rho_s = (float)s;
        rho_d = (float)d;
    }
};

struct Entity : EntityBase {
    std::shared_ptr<Mesh> mesh;
    Entity(const std::string& path, const std::string& type, bool smooth, const py::sequence& c)
        : EntityBase(path, type, smooth, c) {
        mesh = load_mesh(path, type);
    }
};

struct BodyFixedEntity : EntityBase {
    using EntityBase::EntityBase;
};

crt_entity_desc entity_desc(const EntityBase& e, const Mesh& m, uint32_t id) {
    crt_entity_desc d;
    d.tri_xyz = m.xyz.data();
    d.tri_vn = m.vn.empty() ? nullptr : m.vn.data();
    d.n_tris = m.n;
    d.scale = e.scale;
    std::copy(e.position, e.position + 3, d.position);
    std::copy(e.rotation, e.rotation + 9, d.rotation);
    std::copy(e.color, e.color + 3, d.color);
    d.smooth_shading = e.smooth_shading ? 1 : 0;
    d.id = id;
    d.rho_s = e.rho_s;
    d.rho_d = e.rho_d;
    return d;
}

struct SceneHandle {
    crt_scene* s = nullptr;
    SceneHandle() = default;
    SceneHandle(const SceneHandle&) = delete;
    ~SceneHandle() {
        if (s) {
            std::lock_guard<std::mutex> lk(g_mu);
            crt_scene_destroy(s);
        }
    }
};

// sah: -1 the context's setting, 0 radix tree without treelet restructuring (the shortest build),
// 1 binned SAH with the context's treelet passes (for this scene's build only)
std::unique_ptr<SceneHandle> build_scene(const std::vector<crt_entity_desc>& descs, int sah = -1) {
    auto h = std::make_unique<SceneHandle>();
    py::gil_scoped_release nogil;
    std::lock_guard<std::mutex> lk(g_mu);
    crt_tuning saved;
    const bool swap = sah >= 0 && crt_context_get_tuning(ctx(), &saved) == CRT_OK &&
                      (saved.build_sah != sah || (sah == 0 && saved.treelet_passes != 0));
    if (swap) {
        crt_tuning t = saved;
        t.build_sah = sah;
        if (sah == 0) t.treelet_passes = 0;
        crt_context_set_tuning(ctx(), &t);
    }
    int rc = crt_scene_create(ctx(), descs.data(), (uint32_t)descs.size(), &h->s);
    if (swap) crt_context_set_tuning(ctx(), &saved);
    if (rc != CRT_OK) raise_status(rc, "scene build");
    if (verbose()) {
        crt_scene_stats st;
        crt_scene_get_stats(h->s, &st);
        std::printf("    BVH of %zu node(s) and %zu reference(s)\n    BVH built in %g seconds\n", st.n_nodes, st.n_tris,
                    st.build_ms / 1000.0);
    }
    return h;
}

std::vector<crt_light_desc> light_descs(const py::list& lights) {
    std::vector<crt_light_desc> out;
    for (const py::handle& h : lights) {
        crt_light_desc d{};
        if (py::isinstance<PointLight>(h)) {
            const PointLight& l = h.cast<const PointLight&>();
            d.type = 0;
            d.intensity = l.intensity;
            std::copy(l.position, l.position + 3, d.position);
            std::copy(l.rotation, l.rotation + 9, d.rotation);
        } else if (py::isinstance<AreaLight>(h)) {
            const AreaLight& l = h.cast<const AreaLight&>();
            d.type = 1;
            d.intensity = l.intensity;
            std::copy(l.position, l.position + 3, d.position);
            std::copy(l.rotation, l.rotation + 9, d.rotation);
            d.size[0] = l.size[0];
            d.size[1] = l.size[1];
        } else {
            continue;   // the reference skips unknown light types (src/pybind.cpp:476-484)
        }
        out.push_back(d);
    }
    return out;
}

const SimpleCamera& camera_of(const py::handle& h) {
    if (!py::isinstance<SimpleCamera>(h)) throw py::type_error("camera must be a SimpleCamera");
    return h.cast<const SimpleCamera&>();
}
const SimpleLidar& lidar_of(const py::handle& h) {
    if (!py::isinstance<SimpleLidar>(h)) throw py::type_error("lidar must be a SimpleLidar");
    return h.cast<const SimpleLidar&>();
}

// ---------------------------------------------------------------- queries on a built scene
py::object do_render(crt_scene* s, const SimpleCamera& cam, const py::list& lights, int min_s, int max_s, double thr,
                     int bounces, uint64_t seed, uint32_t request, bool return_radiance) {
    const crt_camera_desc cd = cam.desc();
    const auto ls = light_descs(lights);
    crt_render_params p{min_s, max_s, thr, bounces, seed, request};
    py::array_t<uint8_t> img = pinned_array<uint8_t>({cam.height(), cam.width(), 4});
    py::array_t<float> rad;
    if (return_radiance) rad = pinned_array<float>({cam.height(), cam.width(), 4});
    {
        uint8_t* ip = img.mutable_data();
        float* rp = return_radiance ? rad.mutable_data() : nullptr;
        py::gil_scoped_release nogil;
        std::lock_guard<std::mutex> lk(g_mu);
        int rc = crt_render(s, &cd, ls.data(), (uint32_t)ls.size(), &p, ip, rp);
        if (rc != CRT_OK) raise_status(rc, "render");
    }
    if (return_radiance) return py::make_tuple(img, rad);
    return std::move(img);
}

py::array_t<double> do_points(crt_scene* s, const SimpleCamera& cam, bool normals) {
    const crt_camera_desc cd = cam.desc();
    py::array_t<double> out = pinned_array<double>({cam.height(), cam.width(), 3});
    double* o = out.mutable_data();
    py::gil_scoped_release nogil;
    std::lock_guard<std::mutex> lk(g_mu);
    int rc = normals ? crt_passes(s, &cd, nullptr, nullptr, o) : crt_passes(s, &cd, o, nullptr, nullptr);
    if (rc != CRT_OK) raise_status(rc, normals ? "normal_pass" : "intersection_pass");
    return out;
}

py::array_t<uint32_t> do_instances(crt_scene* s, const SimpleCamera& cam) {
    const crt_camera_desc cd = cam.desc();
    py::array_t<uint32_t> out = pinned_array<uint32_t>({cam.height(), cam.width()});
    uint32_t* o = out.mutable_data();
    py::gil_scoped_release nogil;
    std::lock_guard<std::mutex> lk(g_mu);
    int rc = crt_passes(s, &cd, nullptr, o, nullptr);
    if (rc != CRT_OK) raise_status(rc, "instance_pass");
    return out;
}

double do_single_lidar(crt_scene* s, const SimpleLidar& l) {
    double r = 0;
    py::gil_scoped_release nogil;
    std::lock_guard<std::mutex> lk(g_mu);
    int rc = crt_lidar_batch(s, l.position, l.rotation, 1, l.z_positive ? 1 : 0, &r, nullptr);
    if (rc != CRT_OK) raise_status(rc, "simulate_lidar");
    return r;
}

py::array_t<double> do_batch_lidar(crt_scene* s, const SimpleLidar& l) {
    const size_t n = l.batch_positions.size() / 3;
    py::array_t<double> out = pinned_array<double>({(py::ssize_t)1, (py::ssize_t)n});
    double* o = out.mutable_data();
    if (n) {
        py::gil_scoped_release nogil;
        std::lock_guard<std::mutex> lk(g_mu);
        int rc = crt_lidar_batch(s, l.batch_positions.data(), l.batch_rotations.data(), n, l.z_positive ? 1 : 0, o,
                                 nullptr);
        if (rc != CRT_OK) raise_status(rc, "batch_simulate_lidar");
    }
    return out;
}

py::tuple do_lidar_scan(crt_scene* s, const SimpleLidar& l) {
    if (!l.nx || !l.ny) throw py::value_error("lidar has no beam grid: call set_beam_grid first");
    crt_lidar_grid_desc g;
    std::copy(l.position, l.position + 3, g.position);
    std::copy(l.rotation, l.rotation + 9, g.rotation);
    g.z_positive = l.z_positive ? 1 : 0;
    g.nx = l.nx;
    g.ny = l.ny;
    g.half_angle_x = l.half_x;
    g.half_angle_y = l.half_y;
    py::array_t<double> rng = pinned_array<double>({(py::ssize_t)l.ny, (py::ssize_t)l.nx});
    py::array_t<uint32_t> prim = pinned_array<uint32_t>({(py::ssize_t)l.ny, (py::ssize_t)l.nx});
    double* rp = rng.mutable_data();
    uint32_t* pp = prim.mutable_data();
    {
        py::gil_scoped_release nogil;
        std::lock_guard<std::mutex> lk(g_mu);
        int rc = crt_lidar_grid(s, &g, rp, pp);
        if (rc != CRT_OK) raise_status(rc, "lidar_scan");
    }
    return py::make_tuple(rng, prim);
}

// ---------------------------------------------------------------- groups
struct BodyFixedGroup : Pose {
    std::vector<std::shared_ptr<Mesh>> meshes;
    std::unique_ptr<SceneHandle> scene;
    double scale = 1.0;
    size_t n_tris = 0;
    // BodyFixedGroup(list[BodyFixedEntity]) (src/pybind.cpp:107-127): entities re-loaded, ids 1..n,
    // BVH built once and kept resident
    explicit BodyFixedGroup(const py::list& lst) {
        std::vector<crt_entity_desc> descs;
        uint32_t id = 1;
        for (const py::handle& h : lst) {
            const BodyFixedEntity& e = h.cast<const BodyFixedEntity&>();
            auto m = load_mesh(e.geometry_path, e.geometry_type);
            meshes.push_back(m);
            descs.push_back(entity_desc(e, *m, id++));
            n_tris += m->n;
        }
        scene = build_scene(descs);
    }
    void set_scale(double s) { scale = s; }
    crt_scene* sc() const { return scene->s; }
};

// The dynamic path rebuilds the BVH on every call.  The binned-SAH topology with one treelet pass
// costs about 9.5 ns per triangle more to build than the radix tree (2M triangles: 23.7 vs 4.7 ms)
// and saves about 10 % of the traversal, ~0.018 ns of ~0.18 ns per ray, so a call uses it only when
// it traces more than about 500 rays per triangle; `rays` is the call's estimate.
std::unique_ptr<SceneHandle> dynamic_scene(const py::list& entities, bool assign_ids, double rays) {
    std::vector<crt_entity_desc> descs;
    uint32_t id = 1;
    double n_tris = 0;
    for (const py::handle& h : entities) {
        Entity& e = h.cast<Entity&>();
        if (assign_ids) e.id = id++;   // instance_pass / normal_pass renumber (src/pybind.cpp:668-675)
        descs.push_back(entity_desc(e, *e.mesh, e.id));
        n_tris += (double)e.mesh->n;
    }
    return build_scene(descs, rays > 500.0 * n_tris ? 1 : 0);
}

double pixels(const SimpleCamera& c) { return (double)std::max(c.width(), 0) * (double)std::max(c.height(), 0); }

template <class T>
void bind_pose(py::class_<T>& c) {
    c.def("set_position", [](T& self, const py::handle& p) { self.set_position(p); })
        .def("set_rotation", [](T& self, const py::handle& r) { self.set_rotation(r); })
        .def("set_pose", [](T& self, const py::handle& p, const py::handle& r) { self.set_pose(p, r); });
}

}  // namespace

PYBIND11_MODULE(_crt, m) {
    m.doc() = "ceres ray tracer (GB300 ray-query path)";
    m.attr("__gb300__") = true;
    m.def("set_device", [](int d) {
        std::lock_guard<std::mutex> lk(g_mu);
        if (g_ctx) throw std::runtime_error("set_device must be called before the first GPU use");
        g_device = d;
    });
    m.def("synchronize", [] {
        py::gil_scoped_release nogil;
        std::lock_guard<std::mutex> lk(g_mu);
        if (g_ctx) {
            int rc = crt_context_synchronize(g_ctx);
            if (rc != CRT_OK) raise_status(rc, "synchronize");
        }
    });

    py::class_<SimpleCamera> cam(m, "SimpleCamera");
    cam.def(py::init<double, const py::sequence&, const py::sequence&, bool>(), py::arg("focal_length"),
            py::arg("resolution"), py::arg("sensor_size"), py::arg("z_positive"));
    bind_pose(cam);

    py::class_<SimpleLidar> lid(m, "SimpleLidar");
    lid.def(py::init<bool>(), py::arg("z_positive"))
        .def("batch_set_pose", &SimpleLidar::batch_set_pose, py::arg("batch_positions"), py::arg("batch_rotations"),
             py::arg("number_of_poses"))
        .def("set_beam_grid", &SimpleLidar::set_beam_grid, py::arg("nx"), py::arg("ny"), py::arg("half_angle_x"),
             py::arg("half_angle_y"));
    bind_pose(lid);

    py::class_<PointLight> pl(m, "PointLight");
    pl.def(py::init<double>(), py::arg("intensity"));
    bind_pose(pl);

    py::class_<AreaLight> al(m, "AreaLight");
    al.def(py::init<double, const py::sequence&>(), py::arg("intensity"), py::arg("size"));
    bind_pose(al);

    py::class_<Entity> ent(m, "Entity");
    ent.def(py::init<const std::string&, const std::string&, bool, const py::sequence&>(), py::arg("geometry_path"),
            py::arg("geometry_type"), py::arg("smooth_shading"), py::arg("color"))
        .def("set_scale", &Entity::set_scale)
        .def("set_reflectivity", &Entity::set_reflectivity, py::arg("specular"), py::arg("diffuse"))
        .def_property_readonly("num_triangles", [](const Entity& e) { return e.mesh->n; });
    bind_pose(ent);

    py::class_<BodyFixedEntity> bfe(m, "BodyFixedEntity");
    bfe.def(py::init<const std::string&, const std::string&, bool, const py::sequence&>(), py::arg("geometry_path"),
            py::arg("geometry_type"), py::arg("smooth_shading"), py::arg("color"))
        .def("set_scale", &BodyFixedEntity::set_scale)
        .def("set_reflectivity", &BodyFixedEntity::set_reflectivity, py::arg("specular"), py::arg("diffuse"));
    bind_pose(bfe);

    py::class_<BodyFixedGroup> grp(m, "BodyFixedGroup");
    grp.def(py::init<const py::list&>())
        .def("set_scale", &BodyFixedGroup::set_scale)
        .def("render",
             [](BodyFixedGroup& g, const py::handle& camera, const py::list& lights, int min_s, int max_s, double thr,
                int bounces, uint64_t seed, uint32_t request, bool return_radiance) {
                 return do_render(g.sc(), camera_of(camera), lights, min_s, max_s, thr, bounces, seed, request,
                                  return_radiance);
             },
             py::arg("camera"), py::arg("lights"), py::arg("min_samples"), py::arg("max_samples"),
             py::arg("noise_threshold"), py::arg("num_bounces"), py::kw_only(), py::arg("seed") = 0,
             py::arg("request") = 0, py::arg("return_radiance") = false)
        .def("simulate_lidar",
             [](BodyFixedGroup& g, const py::handle& lidar, double) { return do_single_lidar(g.sc(), lidar_of(lidar)); },
             py::arg("lidar"), py::arg("num_rays"))
        .def("batch_simulate_lidar",
             [](BodyFixedGroup& g, const py::handle& lidar, double) { return do_batch_lidar(g.sc(), lidar_of(lidar)); },
             py::arg("lidar"), py::arg("num_rays"))
        .def("lidar_scan", [](BodyFixedGroup& g, const py::handle& lidar) { return do_lidar_scan(g.sc(), lidar_of(lidar)); },
             py::arg("lidar"))
        .def("intersection_pass",
             [](BodyFixedGroup& g, const py::handle& camera) { return do_points(g.sc(), camera_of(camera), false); })
        .def("instance_pass",
             [](BodyFixedGroup& g, const py::handle& camera) { return do_instances(g.sc(), camera_of(camera)); })
        .def("normal_pass",
             [](BodyFixedGroup& g, const py::handle& camera) { return do_points(g.sc(), camera_of(camera), true); })
        .def("srp",
             [](BodyFixedGroup& g, const f64arr& sun_dir, const f64arr& quats, uint32_t grid, uint32_t num_bounces,
                double flux, double c, const py::object& cm, bool facet_power) {
                 crt_srp_desc d;
                 if (sun_dir.size() < 3) throw py::value_error("sun_dir needs 3 values");
                 std::copy(sun_dir.data(), sun_dir.data() + 3, d.sun_dir_inertial);
                 d.center_of_mass[0] = d.center_of_mass[1] = d.center_of_mass[2] = 0.0;
                 if (!cm.is_none()) read3(cm, d.center_of_mass);
                 d.flux = flux;
                 d.c = c;
                 d.grid = grid;
                 d.num_bounces = num_bounces;
                 if (quats.size() % 4) throw py::value_error("quaternions must have shape (n, 4)");
                 const size_t n = (size_t)quats.size() / 4;
                 py::array_t<double> f({(py::ssize_t)n, (py::ssize_t)3}), t({(py::ssize_t)n, (py::ssize_t)3});
                 py::array_t<double> fp;
                 if (facet_power) fp = py::array_t<double>({(py::ssize_t)n, (py::ssize_t)g.n_tris});
                 double *fpp = f.mutable_data(), *tpp = t.mutable_data(), *ppp = facet_power ? fp.mutable_data() : nullptr;
                 const double* q = quats.data();
                 {
                     py::gil_scoped_release nogil;
                     std::lock_guard<std::mutex> lk(g_mu);
                     int rc = crt_srp(g.sc(), &d, q, n, fpp, tpp, ppp);
                     if (rc != CRT_OK) raise_status(rc, "srp");
                 }
                 if (facet_power) return py::tuple(py::make_tuple(f, t, fp));
                 return py::tuple(py::make_tuple(f, t));
             },
             py::arg("sun_dir"), py::arg("quaternions"), py::arg("grid"), py::arg("num_bounces") = 2,
             py::arg("flux") = 1361.0, py::arg("c") = 299792458.0,
             py::arg("center_of_mass") = py::none(), py::arg("facet_power") = false)
        .def("scene_stats", [](BodyFixedGroup& g) {
            crt_scene_stats st;
            crt_scene_get_stats(g.sc(), &st);
            py::dict d;
            d["n_tris"] = st.n_tris;
            d["n_nodes"] = st.n_nodes;
            d["depth"] = st.depth;
            d["build_ms"] = st.build_ms;
            d["device_bytes"] = st.device_bytes;
            return d;
        });
    bind_pose(grp);

    // free functions: the dynamic-scene path rebuilds the BVH on every call (rendering_dynamic/*.hpp)
    m.def("render",
          [](const py::handle& camera, const py::list& lights, const py::list& entities, int min_s, int max_s, double thr,
             int bounces, uint64_t seed, uint32_t request, bool return_radiance) {
              // per camera path: the primary ray, a shadow ray per light at each bounce, a bounce ray
              // between bounces
              const double b = std::max(bounces, 0);
              const double rays = pixels(camera_of(camera)) * std::max(max_s, 1) *
                                  (1.0 + b * (double)lights.size() + std::max(b - 1.0, 0.0));
              auto sc = dynamic_scene(entities, false, rays);
              return do_render(sc->s, camera_of(camera), lights, min_s, max_s, thr, bounces, seed, request,
                               return_radiance);
          },
          py::arg("camera"), py::arg("lights"), py::arg("entities"), py::arg("min_samples"), py::arg("max_samples"),
          py::arg("noise_threshold"), py::arg("num_bounces"), py::kw_only(), py::arg("seed") = 0,
          py::arg("request") = 0, py::arg("return_radiance") = false);
    m.def("simulate_lidar", [](const py::handle& lidar, const py::list& entities, int) {
        auto sc = dynamic_scene(entities, false, 1.0);
        return do_single_lidar(sc->s, lidar_of(lidar));
    });
    m.def("intersection_pass", [](const py::handle& camera, const py::list& entities) {
        auto sc = dynamic_scene(entities, false, pixels(camera_of(camera)));
        return do_points(sc->s, camera_of(camera), false);
    });
    m.def("instance_pass", [](const py::handle& camera, const py::list& entities) {
        auto sc = dynamic_scene(entities, true, pixels(camera_of(camera)));
        return do_instances(sc->s, camera_of(camera));
    });
    m.def("normal_pass", [](const py::handle& camera, const py::list& entities) {
        auto sc = dynamic_scene(entities, true, pixels(camera_of(camera)));
        return do_points(sc->s, camera_of(camera), true);
    });
}
