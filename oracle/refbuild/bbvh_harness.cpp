// Drives the reference CPU plugin bbvh.so (bbvh/main.cpp:97-133) through rta's
// plugin ABI (librta/plugins.cpp:82-85) on rays read from a file, and writes
// the closest hits keyed by the original triangle id.
//
// Oracle build recipe only (test infrastructure): compiled against the
// reference headers with the shims in ./shim, never shipped with the product.
//
// usage: bbvh_harness <plugin.so> <tris.f32> <n> <rays.f32> <nrays> <out.bin> [width]
//   tris.f32  n records of 26 float32 (cuda::simple_triangle layout); the
//             material_index column carries the original triangle id
//   rays.f32  nrays * 7 float32: origin xyz, direction xyz, max_t
//   out.bin   nrays * {float t, beta, gamma; uint32 original id or ~0u}
//             followed by one float: trace milliseconds (raytrav.h:426)
#include "librta/librta.h"

#include <dlfcn.h>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

using namespace rta;

namespace {

class buffer_rays : public ray_generator {
  public:
	const float *src;
	buffer_rays(unsigned w, unsigned h, const float *s) : ray_generator(w, h), src(s) {}
	void generate_rays() override {
		for (unsigned y = 0; y < res_y(); ++y)
			for (unsigned x = 0; x < res_x(); ++x) {
				const float *r = src + 7 * ((size_t)y * res_x() + x);
				*origin(x, y) = make_vec3f(r[0], r[1], r[2]);
				*direction(x, y) = make_vec3f(r[3], r[4], r[5]);
				max_t(x, y) = r[6];
			}
	}
	std::string identification() override { return "oracle buffer rays"; }
	void dont_forget_to_initialize_max_t() override {}
};

typedef primary_intersection_collector<simple_aabb, simple_triangle> collector_t;

template <typename T> T sym(void *h, const char *name) {
	T f = (T)dlsym(h, name);
	if (!f) { fprintf(stderr, "missing symbol %s\n", name); exit(2); }
	return f;
}

std::vector<char> slurp(const char *path) {
	FILE *f = fopen(path, "rb");
	if (!f) { perror(path); exit(2); }
	fseek(f, 0, SEEK_END);
	long sz = ftell(f);
	fseek(f, 0, SEEK_SET);
	std::vector<char> b(sz);
	if (fread(b.data(), 1, sz, f) != (size_t)sz) { perror(path); exit(2); }
	fclose(f);
	return b;
}

} // namespace

int main(int argc, char **argv) {
	if (argc < 7) { fprintf(stderr, "usage: %s plugin tris n rays nrays out\n", argv[0]); return 2; }
	void *h = dlopen(argv[1], RTLD_NOW | RTLD_GLOBAL);
	if (!h) { fprintf(stderr, "dlopen: %s\n", dlerror()); return 2; }
	auto initialize = sym<void (*)()>(h, "initialize");
	auto create = sym<rt_set (*)(basic_flat_triangle_list<simple_triangle> &, int, int)>(h, "create_rt_set");
	sym<char *(*)()>(h, "description");
	sym<int (*)(int, char **)>(h, "parse_cmdline");
	initialize();

	unsigned n = (unsigned)strtoul(argv[3], 0, 10);
	unsigned nrays = (unsigned)strtoul(argv[5], 0, 10);
	std::vector<char> tb = slurp(argv[2]);
	std::vector<char> rb = slurp(argv[4]);
	if (tb.size() != (size_t)n * 104 || rb.size() != (size_t)nrays * 28) {
		fprintf(stderr, "input sizes do not match\n");
		return 2;
	}
	static_assert(sizeof(simple_triangle) == 104, "triangle record");
	basic_flat_triangle_list<simple_triangle> ftl(n);
	memcpy((void *)ftl.triangle, tb.data(), tb.size());

	// rays are laid out as a width x (nrays/width) image; the plugin's OpenMP
	// loop runs over image rows (bbvh/bbvh.h:396)
	unsigned w = argc > 7 ? (unsigned)strtoul(argv[7], 0, 10) : nrays;
	if (w == 0 || nrays % w) { fprintf(stderr, "width must divide nrays\n"); return 2; }
	unsigned hgt = nrays / w;
	rt_set set = create(ftl, (int)w, (int)hgt);
	buffer_rays rays(w, hgt, (const float *)rb.data());
	collector_t hits(w, hgt);
	basic_raytracer<simple_aabb, simple_triangle> *rt = set.basic_rt<simple_aabb, simple_triangle>();
	if (!rt) { fprintf(stderr, "plugin tracer has an unexpected type\n"); return 2; }
	rt->ray_generator(&rays);
	rt->ray_bouncer(&hits);
	set.rt->trace();
	float ms = rt->timings.front();

	basic_acceleration_structure<simple_aabb, simple_triangle> *as = set.basic_as<simple_aabb, simple_triangle>();
	simple_triangle *canon = as->canonical_triangle_ptr();
	FILE *out = fopen(argv[6], "wb");
	for (unsigned i = 0; i < nrays; ++i) {
		const triangle_intersection<simple_triangle> &is = hits.intersection(i % w, i / w);
		uint32_t id = ~0u;
		float rec[3] = {is.t, 0.f, 0.f};
		if (is.valid()) {
			rec[1] = is.beta;
			rec[2] = is.gamma;
			memcpy(&id, &canon[is.ref].material_index, 4);
		}
		fwrite(rec, 4, 3, out);
		fwrite(&id, 4, 1, out);
	}
	fwrite(&ms, 4, 1, out);
	fclose(out);
	as->free_canonical_triangles(canon);
	return 0;
}
