/* No-op stand-in for png++ (image output is not on the traced path). */
#ifndef ORACLE_SHIM_PNGPP_H
#define ORACLE_SHIM_PNGPP_H
#include <string>
namespace png {
struct rgb_pixel { rgb_pixel(unsigned char, unsigned char, unsigned char) {} rgb_pixel() {} };
struct rgba_pixel { rgba_pixel(unsigned char, unsigned char, unsigned char, unsigned char) {} rgba_pixel() {} };
template <typename P> struct image {
	image(unsigned, unsigned) {}
	void set_pixel(unsigned, unsigned, P) {}
	void write(const std::string &) {}
};
}
#endif
