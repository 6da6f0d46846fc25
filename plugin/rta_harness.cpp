// rta_harness.cpp -- a headless stand-in for the rta driver (rta/main.cpp)
// that loads a plugin .so and drives it through rta's plugin interfaces in the
// driver's order, so the drop-in plugin bbvh-gb300.so runs exactly as rta
// would run it:
//
//   dlopen (rta/main.cpp:511-513, librta/plugins.cpp:91-96)
//   initialize(), parse_cmdline(argc, argv), create_rt_set(tris, w, h)
//   rt->ray_bouncer(collector); rt->ray_generator(set.rgen), which must be a
//       cam_ray_generator_shirley (rta/main.cpp:479-488)
//   crgs->setup(pos, dir, up, fovy); rt->trace(); rt->timings.front()
//       (rta/main.cpp:382-405)
//   -R: ctor->build(device ftl) when !expects_host_triangles(), delete the
//       old AS, rt->acceleration_structure(new AS) (rta/main.cpp:389-400)
//   mamo dumps: as->dump_acceleration_structure / dump_primitives
//       (rta/main.cpp:537-541), crgs->dump_rays (rta/main.cpp:384-387)
//
// It also supplies the three librta symbols a CUDA plugin links against
// (librta/cuda.cpp:13, librta/cuda-kernels.cu:24-44 and :50-112): the flag
// plugin_with_cuda_loaded and the two ray-buffer kernels, here through the
// sm_103a library (rta_reset_intersections, rta_setup_shirley_rays).
//
// Built twice: the executable rta_harness, and librta_harness.so, which a
// process loads with RTLD_GLOBAL to provide the librta symbols before it
// loads the plugin itself (rta_harness_main is the executable's main).
//
// usage: rta_harness <plugin.so> <out-prefix> <scene> [<scene> ...] [-- plugin args]
//   scene   binary file: uint32 n, w, h; float fovy; float cam pos[3], dir[3],
//           up[3]; then n triangle records of 26 float32 (simple_triangle).
//           Every scene after the first is a -R rebuild through the
//           constructor with the same w x h; each scene is one traced frame.
//   output  <prefix>.<k>.hits   w*h records {float t, beta, gamma; uint ref}
//           <prefix>.<k>.ids    uint32 n: Morton position -> input triangle id
//                               (the material_index tag of the canonical copy)
//           <prefix>.<k>.bvh/.tri/.ray  the mamo dumps of frame k
//           <prefix>.log        one line per frame: ms, identification strings
// Exit status 0 on success; the plugin itself exits on CUDA errors, as rta's
// plugins do.
#include "librta/librta.h"
#include "librta/cuda.h"

#include <dlfcn.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "rta_gb300.h"

// ---- the librta symbols a CUDA plugin expects from the driver's process ----
namespace rta {
namespace cuda {
bool plugin_with_cuda_loaded = false;
bool using_cuda() { return plugin_with_cuda_loaded; }

void reset_intersections(triangle_intersection<simple_triangle> *last_intersection, uint w, uint h)
{
    if (rta_reset_intersections(last_intersection, w, h, nullptr) != RTA_OK) {
        fprintf(stderr, "GPUassert: reset_intersections: %s\n", rta_last_error());
        exit(2);
    }
}

void setup_shirley_rays(float *dirs, float *orgs, float *maxts, float fovy, float aspect, int w, int h, float3 *dir,
                        float3 *pos, float3 *up, float maxt)
{
    // the kernel's tanf(M_PI*(fovy/2)/180) once on the host
    const float half = fovy / 2.0f;
    const float height = tanf((float)(M_PI * half / 180.0f));
    if (rta_setup_shirley_rays(dirs, orgs, maxts, height, aspect, w, h, &dir->x, &pos->x, &up->x, maxt, nullptr) !=
        RTA_OK) {
        fprintf(stderr, "GPUassert: setup_shirley_rays: %s\n", rta_last_error());
        exit(2);
    }
}
} // namespace cuda
} // namespace rta

using namespace rta;

namespace {

typedef cuda::simple_aabb box_t;
typedef cuda::simple_triangle tri_t;
typedef cuda::primary_intersection_collector<box_t, tri_t> collector_t;

struct scene {
    uint32_t n = 0, w = 0, h = 0;
    float fovy = 60.0f;
    vec3f pos, dir, up;
    std::vector<simple_triangle> tris;
};

bool read_scene(const char *path, scene &s)
{
    FILE *f = fopen(path, "rb");
    if (!f) return false;
    uint32_t hdr[3];
    float cam[10];
    bool ok = fread(hdr, 4, 3, f) == 3 && fread(cam, 4, 10, f) == 10;
    if (ok) {
        s.n = hdr[0];
        s.w = hdr[1];
        s.h = hdr[2];
        s.fovy = cam[0];
        s.pos = make_vec3f(cam[1], cam[2], cam[3]);
        s.dir = make_vec3f(cam[4], cam[5], cam[6]);
        s.up = make_vec3f(cam[7], cam[8], cam[9]);
        s.tris.resize(s.n);
        ok = fread(s.tris.data(), sizeof(simple_triangle), s.n, f) == s.n;
    }
    fclose(f);
    return ok && s.n > 0 && s.w > 0 && s.h > 0;
}

template <typename T> T symbol(void *lib, const char *name)
{
    T f = reinterpret_cast<T>(dlsym(lib, name));
    if (!f) {
        fprintf(stderr, "plugin lacks %s\n", name);
        exit(2);
    }
    return f;
}

bool write_file(const std::string &path, const void *data, size_t bytes)
{
    FILE *f = fopen(path.c_str(), "wb");
    if (!f) return false;
    const bool ok = fwrite(data, 1, bytes, f) == bytes;
    fclose(f);
    return ok;
}

// hits of the collector and the canonical triangles' tags, after one frame
bool write_frame(const std::string &prefix, int k, collector_t &hits,
                 basic_acceleration_structure<box_t, tri_t> *as)
{
    const size_t nh = (size_t)hits.w * hits.h;
    std::vector<triangle_intersection<tri_t>> h(nh);
    if (cudaMemcpy(h.data(), hits.gpu_last_intersection, nh * sizeof(h[0]), cudaMemcpyDeviceToHost) != cudaSuccess)
        return false;
    tri_t *canon = as->canonical_triangle_ptr();
    const int n = as->triangle_count();
    std::vector<uint32_t> ids(n);
    for (int i = 0; i < n; ++i) memcpy(&ids[i], &canon[i].material_index, 4);
    as->free_canonical_triangles(canon);
    const std::string base = prefix + "." + std::to_string(k);
    return write_file(base + ".hits", h.data(), nh * sizeof(h[0])) &&
           write_file(base + ".ids", ids.data(), ids.size() * 4);
}

} // namespace

extern "C" int rta_harness_main(int argc, char **argv)
{
    if (argc < 4) {
        fprintf(stderr, "usage: %s plugin.so out-prefix scene [scene ...] [-- plugin args]\n", argv[0]);
        return 2;
    }
    const std::string prefix = argv[2];
    std::vector<const char *> scene_paths;
    std::vector<char *> plugin_args = {argv[1]};
    int i = 3;
    for (; i < argc && strcmp(argv[i], "--") != 0; ++i) scene_paths.push_back(argv[i]);
    for (++i; i < argc; ++i) plugin_args.push_back(argv[i]);

    // load and set up the plugin as the driver does
    void *lib = dlopen(argv[1], RTLD_LAZY | RTLD_GLOBAL);
    if (!lib) {
        fprintf(stderr, "dlopen: %s\n", dlerror());
        return 2;
    }
    auto description = symbol<char *(*)()>(lib, "description");
    auto initialize = symbol<void (*)()>(lib, "initialize");
    auto parse_cmdline = symbol<int (*)(int, char **)>(lib, "parse_cmdline");
    auto create_rt_set = symbol<rt_set (*)(basic_flat_triangle_list<simple_triangle> &, int, int)>(lib, "create_rt_set");
    initialize();
    if (!cuda::plugin_with_cuda_loaded) {
        fprintf(stderr, "initialize() did not announce a CUDA plugin\n");
        return 3;
    }
    if (parse_cmdline((int)plugin_args.size(), plugin_args.data()) != 0) {
        fprintf(stderr, "parse_cmdline failed\n");
        return 3;
    }

    std::vector<scene> scenes(scene_paths.size());
    for (size_t k = 0; k < scenes.size(); ++k)
        if (!read_scene(scene_paths[k], scenes[k]) || scenes[k].w != scenes[0].w || scenes[k].h != scenes[0].h) {
            fprintf(stderr, "bad scene %s\n", scene_paths[k]);
            return 2;
        }
    const int w = (int)scenes[0].w, h = (int)scenes[0].h;

    // the first scene goes through create_rt_set (host triangles)
    basic_flat_triangle_list<simple_triangle> ftl(scenes[0].n);
    memcpy((void *)ftl.triangle, scenes[0].tris.data(), sizeof(simple_triangle) * scenes[0].n);
    rt_set set = create_rt_set(ftl, w, h);
    auto *rt = set.basic_rt<box_t, tri_t>();
    auto *crgs = dynamic_cast<cam_ray_generator_shirley *>(set.rgen);
    if (!rt || !set.as || !set.ctor || !crgs) {
        fprintf(stderr, "the plugin's rt_set lacks a tracer, AS, constructor or shirley generator\n");
        return 3;
    }
    collector_t hits(w, h);
    rt->ray_bouncer(&hits);
    rt->ray_generator(set.rgen);

    FILE *log = fopen((prefix + ".log").c_str(), "w");
    if (!log) return 2;
    fprintf(log, "description %s\n", description());
    cuda_ftl device_ftl;
    for (size_t k = 0; k < scenes.size(); ++k) {
        scene &s = scenes[k];
        if (k > 0) {
            // -R: rebuild through the constructor and re-bind the tracer
            auto *ctor = set.basic_ctor<box_t, tri_t>();
            cudaFree(device_ftl.triangle);
            device_ftl.triangle = nullptr;
            basic_acceleration_structure<box_t, tri_t> *bas;
            cuda_ftl host_ftl;
            host_ftl.triangles = s.n;
            host_ftl.triangle = reinterpret_cast<tri_t *>(s.tris.data());
            if (ctor->expects_host_triangles()) {
                bas = ctor->build(&host_ftl);
            } else {
                if (cudaMalloc((void **)&device_ftl.triangle, sizeof(tri_t) * s.n) != cudaSuccess ||
                    cudaMemcpy(device_ftl.triangle, s.tris.data(), sizeof(tri_t) * s.n, cudaMemcpyHostToDevice) !=
                        cudaSuccess) {
                    fprintf(stderr, "triangle upload failed\n");
                    return 2;
                }
                device_ftl.triangles = s.n;
                bas = ctor->build(&device_ftl);
            }
            host_ftl.triangle = nullptr;
            delete set.as;
            set.as = bas;
            rt->acceleration_structure(bas);
            if (rt->acceleration_structure() != bas) {
                fprintf(stderr, "the tracer did not take the rebuilt acceleration structure\n");
                return 3;
            }
        }
        crgs->setup(&s.pos, &s.dir, &s.up, s.fovy);
        crgs->generate_rays();
        set.rt->trace();
        if (cudaDeviceSynchronize() != cudaSuccess) return 4;
        auto *as = set.basic_as<box_t, tri_t>();
        if (!write_frame(prefix, (int)k, hits, as)) return 4;
        const std::string base = prefix + "." + std::to_string(k);
        as->dump_acceleration_structure(base + ".bvh");
        as->dump_primitives(base + ".tri");
        crgs->dump_rays(base + ".ray");
        fprintf(log, "frame %zu triangles %u ms %.4f passes %zu as %s rt %s rgen %s\n", k, s.n, rt->timings.front(),
                rt->timings.size(), as->identification().c_str(), set.rt->identification().c_str(),
                set.rgen->identification().c_str());
    }
    fclose(log);
    cudaFree(device_ftl.triangle);
    return 0;
}

#ifndef RTA_HARNESS_LIBRARY
int main(int argc, char **argv) { return rta_harness_main(argc, argv); }
#endif
