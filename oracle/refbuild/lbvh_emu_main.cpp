// Runs the reference's own CUDA code on the CPU (through shim/cudaemu) to
// produce golden data: the LBVH pipeline in the order of
// lbvh_constructor::buildCUDA (bbvh-cuda/lbvh.h:153-211), the 2F4 traversal
// kernels (bbvh-cuda/kernels.cu) and the Shirley ray kernel
// (librta/cuda-kernels.cu:50-112).
//
// Oracle build recipe only (test infrastructure).
//
//   lbvh_emu lbvh  <tris.f32> <n> <out_prefix>
//       writes <p>.codes (u32 n), <p>.ids (u32 n), <p>.nodes ((2n-1)*32 B, 2F4),
//              <p>.tris (n*104 B, permuted), <p>.scene (6 f32)
//   lbvh_emu trace <mode> <nodes> <n> <tris.f32> <rays.f32> <nrays> <out>
//       mode: cis | dis | shadow_cis | shadow_dis | cis_aila | dis_aila
//       rays.f32: nrays*7 f32 (origin, direction, max_t); out: nrays*16 B hits
//       after reset_intersections (cuda-kernels.cu:24-44)
//   lbvh_emu rays <w> <h> <fovy> <pos xyz> <dir xyz> <up xyz> <out>
//       out: w*h*7 f32 (origin, direction, max_t) then 1 f32: the tanf value
#include "bbvh-cuda-node.h"
#include "librta/cuda-kernels.h"

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

namespace rta {
namespace cuda {
void setupCudaMemory(uint **indices, uint **codes, void **nodes, int node_t_size, uint **parents,
                     cuda::simple_aabb **boxes, float3 **centers, cuda::simple_triangle **t_out, int n);
float initTriangles(cuda::simple_triangle *triangles, cuda::simple_triangle *src, simple_aabb *boxes,
                    float3 *centers, int n);
float calculateVoxelBounds(simple_aabb &result, simple_aabb *d_boxes, int n);
float calculateMortonCodes2(float3 *centers, simple_aabb voxel_bounds, uint *d_codes, uint *d_indices, int n);
float sortMortonCodes(uint *d_codes, uint *d_indices, int n);
float buildTreeKarras(cuda::bbvh_node_float4<cuda::simple_aabb> *nodes, uint *d_codes, uint *d_indices,
                      uint *parents, int n);
float buildBoundingBoxesKarras2(cuda::bbvh_node_float4<cuda::simple_aabb> *nodes, simple_aabb *boxes,
                                uint *d_codes, uint *d_indices, uint *parents, int n);
float invert_triangle_permutation_cuda(uint *indices, simple_triangle *triangles, simple_triangle *t_out, int n);

typedef bbvh_node_float4<simple_aabb> node4;
typedef triangle_intersection<simple_triangle> hit_t;
#define TRACE_DECL(name) \
	void name(simple_triangle *, int, node4 *, vec3f *, vec3f *, float *, int, int, hit_t *);
TRACE_DECL(trace_cis)
TRACE_DECL(trace_dis)
TRACE_DECL(trace_shadow_cis)
TRACE_DECL(trace_shadow_dis)
TRACE_DECL(trace_cis_ailabox)
TRACE_DECL(trace_dis_ailabox)
#undef TRACE_DECL
void setup_shirley_rays(float *dirs, float *orgs, float *maxts, float fovy, float aspect, int w, int h,
                        float3 *dir, float3 *pos, float3 *up, float maxt);
} // namespace cuda
} // namespace rta

using namespace rta;

static std::vector<char> slurp(const char *path) {
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

static void spill(const std::string &path, const void *p, size_t n) {
	FILE *f = fopen(path.c_str(), "wb");
	if (!f) { perror(path.c_str()); exit(2); }
	fwrite(p, 1, n, f);
	fclose(f);
}

static int run_lbvh(int argc, char **argv) {
	if (argc < 5) return 2;
	int n = atoi(argv[3]);
	std::string pre = argv[4];
	std::vector<char> tb = slurp(argv[2]);
	if (tb.size() != (size_t)n * sizeof(cuda::simple_triangle)) { fprintf(stderr, "size\n"); return 2; }
	// the caller's device triangle list (lbvh.h:147-150)
	cuda::simple_triangle *input = (cuda::simple_triangle *)malloc(tb.size());
	memcpy(input, tb.data(), tb.size());
	uint *d_indices, *d_codes, *d_parents;
	cuda::node4 *d_nodes;
	cuda::simple_aabb *d_boxes;
	float3 *d_centers;
	cuda::simple_triangle *d_triangles;
	cuda::setupCudaMemory(&d_indices, &d_codes, (void **)&d_nodes, sizeof(cuda::node4), &d_parents, &d_boxes,
	                      &d_centers, &d_triangles, n);
	cuda::simple_aabb bounds;
	cuda::initTriangles(d_triangles, input, d_boxes, d_centers, n);
	cuda::calculateVoxelBounds(bounds, d_boxes, n);
	cuda::calculateMortonCodes2(d_centers, bounds, d_codes, d_indices, n);
	cuda::sortMortonCodes(d_codes, d_indices, n);
	cuda::buildTreeKarras(d_nodes, d_codes, d_indices, d_parents, n);
	cuda::buildBoundingBoxesKarras2(d_nodes, d_boxes, d_codes, d_indices, d_parents, n);
	cuda::invert_triangle_permutation_cuda(d_indices, d_triangles, input, n);
	spill(pre + ".codes", d_codes, (size_t)n * 4);
	spill(pre + ".ids", d_indices, (size_t)n * 4);
	spill(pre + ".nodes", d_nodes, (size_t)(2 * n - 1) * sizeof(cuda::node4));
	spill(pre + ".tris", input, tb.size());
	float sc[6] = {bounds.min.x, bounds.min.y, bounds.min.z, bounds.max.x, bounds.max.y, bounds.max.z};
	spill(pre + ".scene", sc, sizeof(sc));
	return 0;
}

static int run_trace(int argc, char **argv) {
	if (argc < 9) return 2;
	std::string mode = argv[2];
	std::vector<char> nb = slurp(argv[3]);
	int n = atoi(argv[4]);
	std::vector<char> tb = slurp(argv[5]);
	std::vector<char> rb = slurp(argv[6]);
	int nrays = atoi(argv[7]);
	if (rb.size() != (size_t)nrays * 28 || tb.size() != (size_t)n * 104) { fprintf(stderr, "size\n"); return 2; }
	std::vector<vec3f> o(nrays), d(nrays);
	std::vector<float> mt(nrays);
	const float *r = (const float *)rb.data();
	for (int i = 0; i < nrays; ++i) {
		o[i] = make_vec3f(r[7 * i + 0], r[7 * i + 1], r[7 * i + 2]);
		d[i] = make_vec3f(r[7 * i + 3], r[7 * i + 4], r[7 * i + 5]);
		mt[i] = r[7 * i + 6];
	}
	std::vector<cuda::hit_t> hits(nrays);
	memset(hits.data(), 0, hits.size() * sizeof(cuda::hit_t));
	cuda::reset_intersections(hits.data(), nrays, 1);
	cuda::simple_triangle *tris = (cuda::simple_triangle *)tb.data();
	cuda::node4 *nodes = (cuda::node4 *)nb.data();
	void (*fn)(cuda::simple_triangle *, int, cuda::node4 *, vec3f *, vec3f *, float *, int, int, cuda::hit_t *) = 0;
	if (mode == "cis") fn = cuda::trace_cis;
	else if (mode == "dis") fn = cuda::trace_dis;
	else if (mode == "shadow_cis") fn = cuda::trace_shadow_cis;
	else if (mode == "shadow_dis") fn = cuda::trace_shadow_dis;
	else if (mode == "cis_aila") fn = cuda::trace_cis_ailabox;
	else if (mode == "dis_aila") fn = cuda::trace_dis_ailabox;
	else { fprintf(stderr, "mode\n"); return 2; }
	fn(tris, n, nodes, o.data(), d.data(), mt.data(), nrays, 1, hits.data());
	spill(argv[8], hits.data(), hits.size() * sizeof(cuda::hit_t));
	return 0;
}

static int run_rays(int argc, char **argv) {
	if (argc < 15) return 2;
	int w = atoi(argv[2]), h = atoi(argv[3]);
	float fovy = (float)atof(argv[4]);
	float3 pos = make_float3((float)atof(argv[5]), (float)atof(argv[6]), (float)atof(argv[7]));
	float3 dir = make_float3((float)atof(argv[8]), (float)atof(argv[9]), (float)atof(argv[10]));
	float3 up = make_float3((float)atof(argv[11]), (float)atof(argv[12]), (float)atof(argv[13]));
	// aspect as the reference's camera computes it (raytrav.h:336)
	float aspect = float(w) / float(h);
	std::vector<float> dirs(3 * (size_t)w * h), orgs(3 * (size_t)w * h), maxts((size_t)w * h);
	cuda::setup_shirley_rays(dirs.data(), orgs.data(), maxts.data(), fovy, aspect, w, h, &dir, &pos, &up, FLT_MAX);
	std::vector<float> out(7 * (size_t)w * h + 1);
	for (size_t i = 0; i < (size_t)w * h; ++i) {
		for (int k = 0; k < 3; ++k) {
			out[7 * i + k] = orgs[3 * i + k];
			out[7 * i + 3 + k] = dirs[3 * i + k];
		}
		out[7 * i + 6] = maxts[i];
	}
	float half = fovy;
	half /= 2.0;
	out.back() = tanf(M_PI * half / 180.0f);
	spill(argv[14], out.data(), out.size() * 4);
	return 0;
}

int main(int argc, char **argv) {
	if (argc < 2) return 2;
	std::string cmd = argv[1];
	if (cmd == "lbvh") return run_lbvh(argc, argv);
	if (cmd == "trace") return run_trace(argc, argv);
	if (cmd == "rays") return run_rays(argc, argv);
	return 2;
}
