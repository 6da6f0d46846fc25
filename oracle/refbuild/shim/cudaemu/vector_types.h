/* CPU stand-in for CUDA's vector types, used only to run the reference's
 * kernels on the host for the checker (oracle build recipe). */
#ifndef ORACLE_EMU_VECTOR_TYPES_H
#define ORACLE_EMU_VECTOR_TYPES_H
typedef unsigned int uint;
struct float2 { float x, y; } __attribute__((aligned(8)));
struct float3 { float x, y, z; };
struct float4 { float x, y, z, w; } __attribute__((aligned(16)));
struct int2 { int x, y; } __attribute__((aligned(8)));
struct uint3 { unsigned x, y, z; };
struct dim3 {
	unsigned x, y, z;
	dim3(unsigned vx = 1, unsigned vy = 1, unsigned vz = 1) : x(vx), y(vy), z(vz) {}
};
static inline float2 make_float2(float x, float y) { float2 r; r.x = x; r.y = y; return r; }
static inline float3 make_float3(float x, float y, float z) { float3 r; r.x = x; r.y = y; r.z = z; return r; }
static inline float4 make_float4(float x, float y, float z, float w) { float4 r; r.x = x; r.y = y; r.z = z; r.w = w; return r; }
static inline int2 make_int2(int x, int y) { int2 r; r.x = x; r.y = y; return r; }
#endif
