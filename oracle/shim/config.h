/* Minimal stand-in for the configure-generated config.h that the
 * reference's stdinc.h includes: a hosted C99 system with standard headers. */
#define STDC_HEADERS 1
#define HAVE_LIMITS_H 1
