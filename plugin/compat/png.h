/* Empty stand-in for <png.h>: the reference's image.h includes it, the traced
 * path never writes an image.  Oracle build recipe only. */
