/* Hand-written configuration for compiling the reference ngspice transient
 * path (analysis, NI, KLU, R/C/V/I/D/MOS1/BSIM4 devices, INP parser) as a
 * test oracle.  Mirrors the default autotools build: KLU and XSPICE on,
 * PREDICTOR off, no X11, no readline. */
#ifndef NGSPICE_CONFIG_H
#define NGSPICE_CONFIG_H
#define PACKAGE "ngspice"
#define PACKAGE_VERSION "46"
#define VERSION "46"
#define NGSPICEBUILDDATE "oracle"
#define STDC_HEADERS 1
#define HAVE_STDLIB_H 1
#define HAVE_STRING_H 1
#define HAVE_STRINGS_H 1
#define HAVE_UNISTD_H 1
#define HAVE_CTYPE_H 1
#define HAVE_LIMITS_H 1
#define HAVE_FLOAT_H 1
#define HAVE_SYS_TYPES_H 1
#define HAVE_SYS_TIME_H 1
#define HAVE_TIME_H 1
#define HAVE_DIRENT_H 1
#define HAVE_FCNTL_H 1
#define HAVE_STRCHR 1
#define HAVE_STRRCHR 1
#define HAVE_STRDUP 1
#define HAVE_GETRUSAGE 1
#define HAVE_GETTIMEOFDAY 1
#define HAVE_ISNAN 1
#define HAVE_ISINF 1
#define HAVE_ERFC 1
#define HAVE_LOGB 1
#define HAVE_SCALBN 1
#define HAVE_DECL_ISNAN 1
#define HAVE_DECL_ISINF 1
#define HAVE_LOCALE_H 1
#define X_DISPLAY_MISSING 1
#define KLU 1
#define XSPICE 1
#define USE_OMP 1
#endif
