// bbvh_gb300.cpp -- rta plugin: a drop-in for bbvh-cuda whose LBVH builder and
// tracers run the sm_103a kernels of librta_gb300 (include/rta_gb300.h).
//
// Same plugin ABI as the reference (librta/plugins.cpp:82-85): description,
// initialize, parse_cmdline, create_rt_set; same command line as bbvh-cuda
// (bbvh-cuda/main.cpp:40-51) plus --morton-bits.  The objects it returns
// implement librta's interfaces:
//   lbvh_ctor  basic_acceleration_structure_constructor, expects device triangles
//              (lbvh_constructor, bbvh-cuda/lbvh.h:49-216)
//   lbvh_as    basic_acceleration_structure; triangle_ptr() is the
//              Morton-ordered triangle array that triangle_intersection::ref
//              indexes, index_buffer maps it to input ids (lbvh.h:13-34)
//   tracer     cuda::gpu_raytracer with the acceleration_structure() re-binding
//              override (bbvh-cuda/bbvh-cuda.h:79-94); -t/-s/-A pick the mode
//   shirley    cuda::cam_ray_generator_shirley whose rays come from
//              rta_setup_shirley_rays (librta/cuda.h:146-158)
// A failing C-ABI call prints the library's message and exits, which is the
// reference's error behaviour (checked_cuda, librta/cuda.h:70-77).
#include "librta/librta.h"
#include "librta/cuda.h"
#include "librta/wall-timer.h"

#include <argp.h>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <string>
#include <vector>

#include "rta_gb300.h"

using namespace rta;

namespace gb300 {

typedef cuda::simple_aabb box_t;
typedef cuda::simple_triangle tri_t;

static void checked(int rc, const char *what)
{
    if (rc != RTA_OK) {
        fprintf(stderr, "GPUassert: %s failed (%d): %s\n", what, rc, rta_last_error());
        exit(rc < 0 ? -rc : rc);
    }
}

struct options {
    bool verbose = false;
    bool dis = false;
    bool shadow = false;
    bool ailabox = false;
    int morton_bits = 30;
};
static options cmd;

class lbvh_as : public basic_acceleration_structure<box_t, tri_t> {
  public:
    rta_lbvh view;
    tri_t *sorted;   // owned by the constructor, reused across builds
    lbvh_as(const rta_lbvh &v, tri_t *s) : view(v), sorted(s) {}
    std::string identification() override { return "lbvh on gb300 (sm_103a kernels)"; }
    tri_t *triangle_ptr() override { return sorted; }
    int triangle_count() override { return (int)view.n; }
    tri_t *canonical_triangle_ptr() override
    {
        tri_t *t = new tri_t[view.n];
        cudaMemcpy(t, sorted, sizeof(tri_t) * view.n, cudaMemcpyDeviceToHost);
        return t;
    }
    void free_canonical_triangles(tri_t *data) override { delete[] data; }
    std::vector<uint32_t> index_buffer()
    {
        std::vector<uint32_t> ids(view.n);
        cudaMemcpy(ids.data(), view.index, 4 * (size_t)view.n, cudaMemcpyDeviceToHost);
        return ids;
    }
    // mamo triangle dump in the layout of binary_bvh::dump_primitives
    // (bbvh/bbvh.h:53-65): positions and normals of the Morton-ordered records
    void dump_primitives(const std::string &filename) override
    {
        tri_t *t = canonical_triangle_ptr();
        std::ofstream out(filename.c_str());
        out << "tri\n" << view.n << "\n";
        for (uint32_t i = 0; i < view.n; ++i) {
            const tri_t &q = t[i];
            out << i << " " << q.a.x << " " << q.a.y << " " << q.a.z << " " << q.b.x << " " << q.b.y << " " << q.b.z
                << " " << q.c.x << " " << q.c.y << " " << q.c.z << " " << q.na.x << " " << q.na.y << " " << q.na.z
                << " " << q.nb.x << " " << q.nb.y << " " << q.nb.z << " " << q.nc.x << " " << q.nc.y << " " << q.nc.z
                << "\n";
        }
        free_canonical_triangles(t);
    }
    // mamo dump in the layout of binary_bvh::dump_acceleration_structure (bbvh/bbvh.h:36-52)
    void dump_acceleration_structure(const std::string &filename) override
    {
        const size_t nn = 2 * (size_t)view.n - 1;
        float *d = nullptr;
        cudaMalloc(&d, nn * 32);
        checked(rta_lbvh_to_2f4(&view, d, nullptr), "rta_lbvh_to_2f4");
        std::vector<float> h(nn * 8);
        cudaMemcpy(h.data(), d, nn * 32, cudaMemcpyDeviceToHost);
        cudaFree(d);
        std::ofstream out(filename.c_str());
        out << "bvh\n" << nn << "\n";
        for (size_t i = 0; i < nn; ++i) {
            uint32_t w0, w1;
            memcpy(&w0, &h[8 * i], 4);
            memcpy(&w1, &h[8 * i + 1], 4);
            bool inner = (w0 & 1u) == 1u;
            out << i << (inner ? " I " : " L ");
            for (int k = 2; k < 8; ++k) out << h[8 * i + k] << " ";
            if (inner)
                out << 0 << " " << (w0 >> 1) << " " << w1 << "\n";
            else {
                out << (w0 >> 1);
                for (uint32_t j = 0; j < (w0 >> 1); ++j) out << " " << w1 + j;
                out << "\n";
            }
        }
    }
};

class lbvh_ctor : public basic_acceleration_structure_constructor<box_t, tri_t> {
    rta_lbvh_ctx *ctx = nullptr;
    tri_t *sorted = nullptr;
    uint32_t cap = 0;

  public:
    int morton_bits;
    explicit lbvh_ctor(int bits) : morton_bits(bits)
    {
        checked(rta_lbvh_create(&ctx), "rta_lbvh_create");
        if (cmd.verbose) checked(rta_lbvh_set_timing(ctx, 1), "rta_lbvh_set_timing");
    }
    ~lbvh_ctor() override
    {
        rta_lbvh_destroy(ctx);
        cudaFree(sorted);
    }
    std::string identification() override { return "lbvh constructor (gb300)"; }
    bool expects_host_triangles() override { return false; }
    basic_acceleration_structure<box_t, tri_t> *build(cuda_ftl *tris) override
    {
        const uint32_t n = tris->triangles;
        if (n > cap) {
            cudaFree(sorted);
            if (cudaMalloc((void **)&sorted, sizeof(tri_t) * n) != cudaSuccess) {
                fprintf(stderr, "GPUassert: out of memory for %u triangles\n", n);
                exit(2);
            }
            cap = n;
        }
        if (cmd.verbose) {
            std::cout << "Triangles: " << n << std::endl;
            std::cout << "Building BVH on GPU..." << std::endl;
        }
        checked(rta_lbvh_build(ctx, tris->triangle, n, morton_bits, sorted, nullptr), "rta_lbvh_build");
        rta_lbvh v;
        checked(rta_lbvh_get(ctx, &v), "rta_lbvh_get");
        if (cmd.verbose) {
            // the per-pass report of lbvh_constructor::buildCUDA (lbvh.h:172-204);
            // the scene box is folded into the first pass and the triangle
            // permutation into the last
            float ms[RTA_LBVH_PASSES];
            checked(rta_lbvh_pass_ms(ctx, ms), "rta_lbvh_pass_ms");
            uint32_t flags = 0;
            checked(rta_lbvh_status(&v, nullptr, &flags), "rta_lbvh_status");
            std::cout << "=========================================================" << std::endl;
            std::cout << "Time for initializing Triangles and Voxel Bounds: " << ms[0] << " ms" << std::endl;
            std::cout << "Time for calculating Morton Codes: " << ms[1] << " ms" << std::endl;
            std::cout << "Time for sorting Morton Codes: " << ms[2] << " ms" << std::endl;
            std::cout << "Time for tree construction: " << ms[3] << " ms" << std::endl;
            std::cout << "Time for building the bounding boxes and permuting the triangles: " << ms[4] << " ms"
                      << std::endl;
            std::cout << "BVH finished. Total time: " << ms[0] + ms[1] + ms[2] + ms[3] + ms[4] << " ms (device flags "
                      << flags << ")" << std::endl;
            std::cout << "=========================================================" << std::endl;
        }
        return new lbvh_as(v, sorted);
    }
};

class tracer : public cuda::gpu_raytracer<box_t, tri_t> {
  public:
    lbvh_as *bvh;
    uint32_t mode;
    tracer(rta::ray_generator *gen, lbvh_as *as, rta::bouncer *b, uint32_t m)
        : cuda::gpu_raytracer<box_t, tri_t>(gen, b, as), bvh(as), mode(m) {}
    std::string identification() override { return "cuda bbvh tracer (gb300)"; }
    bool supports_max_t() override { return true; }
    tracer *copy() override { return new tracer(*this); }
    void acceleration_structure(basic_acceleration_structure<box_t, tri_t> *as) override
    {
        bvh = dynamic_cast<lbvh_as *>(as);
        cuda::gpu_raytracer<box_t, tri_t>::acceleration_structure(as);
    }
    void prepare_trace() override
    {
        checked(rta_reset_intersections(this->gpu_bouncer->gpu_last_intersection, this->gpu_bouncer->w,
                                        this->gpu_bouncer->h, nullptr),
                "rta_reset_intersections");
    }
    float trace_rays() override
    {
        // timed like the reference's tracers: wall clock around launch + sync
        // (bbvh-cuda/bbvh-cuda.h:108-117)
        wall_time_timer wtt;
        wtt.start();
        const uint32_t n = this->gpu_raygen->w * this->gpu_raygen->h;
        checked(rta_trace(&bvh->view, this->gpu_raygen->gpu_origin, this->gpu_raygen->gpu_direction,
                          this->gpu_raygen->gpu_maxt, n, nullptr, this->gpu_bouncer->gpu_last_intersection,
                          mode, nullptr, nullptr),
                "rta_trace");
        cudaDeviceSynchronize();
        return (float)wtt.look();
    }
};

class shirley : public cuda::cam_ray_generator_shirley {
  public:
    shirley(uint w, uint h) : cuda::cam_ray_generator_shirley(w, h) {}
    void generate_rays() override
    {
        // the per-frame constant of setup_shirley_rays (cuda-kernels.cu:63-64)
        float half = fovy;
        half /= 2.0;
        const float height = tanf(M_PI * half / 180.0f);
        checked(rta_setup_shirley_rays(gpu_direction, gpu_origin, gpu_maxt, height, aspect, (int)w, (int)h,
                                       &dir.x, &position.x, &up.x, FLT_MAX, nullptr),
                "rta_setup_shirley_rays");
        cudaDeviceSynchronize();
    }
    std::string identification() override { return "cuda shirley ray generator (gb300)"; }
    // mamo ray dump in the layout of cam_ray_generator_shirley::dump_rays
    // (librta/raytrav.h:353-366), of the rays on the device (the CPU-side
    // ray image the reference's CUDA generator inherits is never filled)
    void dump_rays(const std::string &filename) override
    {
        const size_t n = (size_t)w * h;
        std::vector<float> o(3 * n), d(3 * n), m(n);
        cudaMemcpy(o.data(), gpu_origin, 12 * n, cudaMemcpyDeviceToHost);
        cudaMemcpy(d.data(), gpu_direction, 12 * n, cudaMemcpyDeviceToHost);
        cudaMemcpy(m.data(), gpu_maxt, 4 * n, cudaMemcpyDeviceToHost);
        std::ofstream out(filename.c_str());
        const int iw = (int)w, ih = (int)h;
        out << "ray\n" << iw << " " << ih << "\n";
        for (int y = 0; y < ih; ++y)
            for (int x = 0; x < iw; ++x) {
                const size_t i = (size_t)y * iw + x;
                out << y * iw + x << " " << 2 << " " << o[3 * i] << " " << o[3 * i + 1] << " " << o[3 * i + 2] << " "
                    << d[3 * i] << " " << d[3 * i + 1] << " " << d[3 * i + 2] << " "
                    << "0 " << m[i] << "\n";
            }
    }
};

} // namespace gb300

// --------------------------------------------------------------------------
// command line (bbvh-cuda/main.cpp:40-109)
// --------------------------------------------------------------------------

static char plugin_name[] = "bbvh-gb300";
static char doc[] = "bbvh-gb300: a rta plugin with an sm_103a LBVH builder and tracer.";
static char args_doc[] = "";
enum { OPT_MORTON = 300 };
static struct argp_option options[] = {
    {"verbose", 'v', 0, 0, "Be verbose."},
    {"bvh", 'b', "<median|lbvh>", 0, "Accepted for compatibility; the tree is always an LBVH."},
    {"layout", 'l', "<cpu|2f4>", 0, "Accepted for compatibility; the node layout is gb300's."},
    {"shadow", 's', 0, 0, "Use the shadow tracer, i.e. early out at first triangle intersection."},
    {"trav", 't', "<dis|cis>", 0, "Traverse dis/cis. Default: cis."},
    {"ailabox", 'A', 0, 0, "Use the box intersection method found in Aila et al's implementation."},
    {"morton-bits", OPT_MORTON, "<30|63>", 0, "Morton code length. Default: 30."},
    {0}};

static error_t parse_options(int key, char *arg, argp_state *state)
{
    std::string sarg = arg ? arg : "";
    switch (key) {
    case 'v': gb300::cmd.verbose = true; break;
    case 't':
        if (sarg == "dis") gb300::cmd.dis = true;
        else if (sarg == "cis") gb300::cmd.dis = false;
        else {
            std::cerr << "Unknown bvh traversal scheme: " << sarg << std::endl;
            argp_usage(state);
        }
        break;
    case 'b': case 'l': break;
    case 's': gb300::cmd.shadow = true; break;
    case 'A': gb300::cmd.ailabox = true; break;
    case OPT_MORTON:
        gb300::cmd.morton_bits = atoi(arg);
        if (gb300::cmd.morton_bits != 30 && gb300::cmd.morton_bits != 63) argp_usage(state);
        break;
    default: return ARGP_ERR_UNKNOWN;
    }
    return 0;
}
static struct argp parser = {options, parse_options, args_doc, doc};

extern "C" {

char *description() { return (char *)"a binary bvh ray tracer (sm_103a lbvh)"; }

void initialize() { rta::cuda::plugin_with_cuda_loaded = true; }

int parse_cmdline(int argc, char **argv)
{
    argv[0] = plugin_name;
    return argp_parse(&parser, argc, argv, 0, 0, 0);
}

rt_set create_rt_set(basic_flat_triangle_list<simple_triangle> &triangle_lists, int w, int h)
{
    using namespace gb300;
    cuda_ftl host(triangle_lists);
    cuda_ftl dev;
    const size_t bytes = sizeof(tri_t) * host.triangles;
    if (cudaMalloc((void **)&dev.triangle, bytes) != cudaSuccess ||
        cudaMemcpy(dev.triangle, host.triangle, bytes, cudaMemcpyHostToDevice) != cudaSuccess) {
        fprintf(stderr, "GPUassert: triangle upload failed\n");
        exit(2);
    }
    dev.triangles = host.triangles;
    lbvh_ctor *ctor = new lbvh_ctor(cmd.morton_bits);
    lbvh_as *as = static_cast<lbvh_as *>(ctor->build(&dev));
    cudaFree(dev.triangle);   // the tree keeps its own Morton-ordered copy
    uint32_t mode = (cmd.dis ? RTA_TRACE_DIS : RTA_TRACE_CIS) | (cmd.shadow ? RTA_TRACE_SHADOW : 0u) |
                    (cmd.ailabox ? RTA_TRACE_AILA : 0u);
    rt_set set;
    set.as = as;
    set.ctor = ctor;
    set.rt = new tracer(0, as, 0, mode);
    set.rgen = new shirley(w, h);
    return set;
}

} // extern "C"
