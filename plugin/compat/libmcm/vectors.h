/* Stand-in for the absent libmcm <libmcm/vectors.h> (rta's basic_types.h:7).
 * Plain float vectors and the component-wise operations the reference CPU code
 * calls, evaluated in the operation order of librta/cuda-vec.h:157-193.
 * Used to compile code against the reference headers (plugin/, oracle recipe). */
#ifndef ORACLE_SHIM_LIBMCM_VECTORS_H
#define ORACLE_SHIM_LIBMCM_VECTORS_H
#include <math.h>
#include <ostream>

struct vec2f { float x, y; };
struct vec3f { float x, y, z; };
struct vec4f { float x, y, z, w; };

inline vec3f make_vec3f(float x, float y, float z) { vec3f v; v.x = x; v.y = y; v.z = z; return v; }
inline vec2f make_vec2f(float x, float y) { vec2f v; v.x = x; v.y = y; return v; }

inline void sub_components_vec3f(vec3f *o, const vec3f *l, const vec3f *r) { o->x = l->x - r->x; o->y = l->y - r->y; o->z = l->z - r->z; }
inline void add_components_vec3f(vec3f *o, const vec3f *l, const vec3f *r) { o->x = l->x + r->x; o->y = l->y + r->y; o->z = l->z + r->z; }
inline void mul_vec3f_by_scalar(vec3f *o, const vec3f *l, float s) { o->x = l->x * s; o->y = l->y * s; o->z = l->z * s; }
inline void div_vec3f_by_scalar(vec3f *o, const vec3f *l, float s) { o->x = l->x / s; o->y = l->y / s; o->z = l->z / s; }
inline float dot_vec3f(const vec3f *l, const vec3f *r) { float s = l->x * r->x; s = s + l->y * r->y; s = s + l->z * r->z; return s; }
inline float length_of_vec3f(const vec3f *v) { return sqrtf(dot_vec3f(v, v)); }
inline void normalize_vec3f(vec3f *v) { float l = length_of_vec3f(v); div_vec3f_by_scalar(v, v, l); }
inline void cross_vec3f(vec3f *o, const vec3f *l, const vec3f *r) {
	float x = (l->y * r->z) - (l->z * r->y);
	float y = (l->z * r->x) - (l->x * r->z);
	float z = (l->x * r->y) - (l->y * r->x);
	o->x = x; o->y = y; o->z = z;
}
inline void sub_components_vec2f(vec2f *o, const vec2f *l, const vec2f *r) { o->x = l->x - r->x; o->y = l->y - r->y; }
inline void add_components_vec2f(vec2f *o, const vec2f *l, const vec2f *r) { o->x = l->x + r->x; o->y = l->y + r->y; }
inline void mul_vec2f_by_scalar(vec2f *o, const vec2f *l, float s) { o->x = l->x * s; o->y = l->y * s; }

inline std::ostream &operator<<(std::ostream &o, const vec3f &v) { return o << "(vec " << v.x << " " << v.y << " " << v.z << ")"; }
#endif
