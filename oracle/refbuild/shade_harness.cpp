// Runs the reference's host shading, lighting_collector::shade and ::reset
// (librta/raytrav.h:174-243), on closest hits and Morton-ordered triangles
// read from files, and writes the 8-bit RGB image it produces.
//
// Oracle build recipe only (test infrastructure): compiled against the
// reference headers with the shims in ../../plugin/compat, never shipped with
// the product.
//
// usage: shade_harness <tris.f32> <n> <hits.bin> <w> <h> <lights.f32> <nlights>
//                      <binary 0|1> <bg_r> <bg_g> <bg_b> <out.rgb>
//   tris.f32    n records of 26 float32 (cuda::simple_triangle layout), in the
//               order the hits' ref indexes
//   hits.bin    w*h records {float t, beta, gamma; uint32 ref}
//   lights.f32  nlights * 6 float32: position xyz, colour rgb
//   out.rgb     w*h*3 bytes, row-major, as image<unsigned char, 3> holds them
#include "librta/librta.h"

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

using namespace rta;

namespace {

class collector : public lighting_collector<simple_aabb, simple_triangle> {
  public:
	collector(unsigned w, unsigned h, image<triangle_intersection<simple_triangle>, 1> *li)
	: lighting_collector<simple_aabb, simple_triangle>(w, h, li) {}
	const unsigned char *pixels() const { return res.data; }
};

std::vector<char> slurp(const char *path) {
	FILE *f = fopen(path, "rb");
	if (!f) { perror(path); exit(2); }
	fseek(f, 0, SEEK_END);
	long sz = ftell(f);
	fseek(f, 0, SEEK_SET);
	std::vector<char> b(sz);
	if (sz && fread(b.data(), 1, sz, f) != (size_t)sz) { perror(path); exit(2); }
	fclose(f);
	return b;
}

} // namespace

int main(int argc, char **argv) {
	if (argc != 13) {
		fprintf(stderr, "usage: %s tris n hits w h lights nlights binary bg_r bg_g bg_b out\n", argv[0]);
		return 2;
	}
	const unsigned n = (unsigned)atol(argv[2]);
	const unsigned w = (unsigned)atol(argv[4]), h = (unsigned)atol(argv[5]);
	const unsigned nl = (unsigned)atol(argv[7]);
	const bool binary = atoi(argv[8]) != 0;
	std::vector<char> tb = slurp(argv[1]), hb = slurp(argv[3]), lb = slurp(argv[6]);
	if (tb.size() != (size_t)n * sizeof(simple_triangle) || hb.size() != (size_t)w * h * 16 ||
	    lb.size() != (size_t)nl * 24) {
		fprintf(stderr, "input sizes do not match\n");
		return 2;
	}
	std::vector<simple_triangle> tris(n);
	memcpy(tris.data(), tb.data(), tb.size());
	image<triangle_intersection<simple_triangle>, 1> li(w, h);
	for (unsigned y = 0; y < h; ++y)
		for (unsigned x = 0; x < w; ++x) {
			const char *r = hb.data() + 16 * ((size_t)y * w + x);
			triangle_intersection<simple_triangle> &is = li.pixel(x, y);
			memcpy(&is.t, r + 0, 4);
			memcpy(&is.beta, r + 4, 4);
			memcpy(&is.gamma, r + 8, 4);
			memcpy(&is.ref, r + 12, 4);
		}
	collector c(w, h, &li);
	c.triangle_ptr(tris.data());
	c.reset(make_vec3f((float)atof(argv[9]), (float)atof(argv[10]), (float)atof(argv[11])));
	const float *L = reinterpret_cast<const float *>(lb.data());
	for (unsigned i = 0; i < nl; ++i)
		c.add_pointlight(make_vec3f(L[6 * i + 0], L[6 * i + 1], L[6 * i + 2]),
		                 make_vec3f(L[6 * i + 3], L[6 * i + 4], L[6 * i + 5]));
	c.shade(binary);
	FILE *o = fopen(argv[12], "wb");
	if (!o) { perror(argv[12]); return 2; }
	fwrite(c.pixels(), 1, (size_t)w * h * 3, o);
	fclose(o);
	return 0;
}
