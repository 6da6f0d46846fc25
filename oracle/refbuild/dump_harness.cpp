// Runs the reference's own mamo text dumps on given arrays, for the checker
// (test infrastructure, compiled against the reference headers by the
// Makefile beside it; never shipped):
//   binary_bvh::dump_acceleration_structure, ::dump_primitives (bbvh/bbvh.h:36-65)
//   cam_ray_generator_shirley::dump_rays (librta/raytrav.h:353-366)
//
// usage: dump_harness <nodes.f32> <nn> <tris.f32> <n> <rays.f32> <w> <h> <out-prefix>
//   nodes.f32  nn records of 8 float32 in the 2F4 layout (bbvh-cuda-node.h:
//              word0 = left<<1|1 or count<<1, word1 = right or first
//              triangle, then box min xyz, max xyz); they fill bbvh_node's
//              type_left_elems, right_tris and box (bbvh/bbvh-node.h:5-43)
//   tris.f32   n records of 26 float32 (simple_triangle)
//   rays.f32   w*h * 7 float32: origin xyz, direction xyz, max_t
//   out        <prefix>.bvh, <prefix>.tri, <prefix>.ray
#include "bbvh/bbvh.h"

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

using namespace rta;

namespace {

std::vector<float> slurp(const char *path, size_t floats)
{
    std::vector<float> v(floats);
    FILE *f = fopen(path, "rb");
    if (!f || fread(v.data(), 4, floats, f) != floats) {
        fprintf(stderr, "cannot read %zu floats from %s\n", floats, path);
        exit(2);
    }
    fclose(f);
    return v;
}

class buffer_shirley : public cam_ray_generator_shirley {
  public:
    buffer_shirley(unsigned w, unsigned h, const float *r) : cam_ray_generator_shirley(w, h)
    {
        for (unsigned y = 0; y < h; ++y)
            for (unsigned x = 0; x < w; ++x) {
                const float *q = r + 7 * ((size_t)y * w + x);
                *origin(x, y) = make_vec3f(q[0], q[1], q[2]);
                *direction(x, y) = make_vec3f(q[3], q[4], q[5]);
                max_t(x, y) = q[6];
            }
    }
    void generate_rays() override {}
};

} // namespace

int main(int argc, char **argv)
{
    if (argc != 9) {
        fprintf(stderr, "usage: %s nodes nn tris n rays w h prefix\n", argv[0]);
        return 2;
    }
    const size_t nn = strtoul(argv[2], 0, 10), n = strtoul(argv[4], 0, 10);
    const unsigned w = (unsigned)strtoul(argv[6], 0, 10), h = (unsigned)strtoul(argv[7], 0, 10);
    const std::string prefix = argv[8];
    std::vector<float> nodes = slurp(argv[1], nn * 8), tris = slurp(argv[3], n * 26),
                       rays = slurp(argv[5], (size_t)w * h * 7);

    binary_bvh<simple_aabb, simple_triangle> bvh;
    bvh.nodes.resize(nn);
    for (size_t i = 0; i < nn; ++i) {
        const float *q = &nodes[8 * i];
        memcpy(&bvh.nodes[i].type_left_elems, q + 0, 4);
        memcpy(&bvh.nodes[i].right_tris, q + 1, 4);
        bvh.nodes[i].box.min = make_vec3f(q[2], q[3], q[4]);
        bvh.nodes[i].box.max = make_vec3f(q[5], q[6], q[7]);
    }
    static_assert(sizeof(simple_triangle) == 104, "triangle record");
    bvh.triangles.resize(n);
    memcpy((void *)bvh.triangles.data(), tris.data(), n * 104);
    bvh.dump_acceleration_structure(prefix + ".bvh");
    bvh.dump_primitives(prefix + ".tri");

    buffer_shirley gen(w, h, rays.data());
    gen.dump_rays(prefix + ".ray");
    return 0;
}
