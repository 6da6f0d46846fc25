/* configure-generated header of the reference, written for builds against the reference headers:
 * RTA_HAVE_LIBCUDART=1. */
#ifndef ORACLE_SHIM_RTA_CONFIG_H
#define ORACLE_SHIM_RTA_CONFIG_H
#define RTA_HAVE_LIBCUDART 1
#define RTA_HAVE_LIBLUMOCL 0
#endif
