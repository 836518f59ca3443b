/* Project-written stand-in for the autoconf-generated config.h of the
 * reference. Only the macros the membrane-surface path tests are set. */
#define HAVE_MATH_H 1
#define HAVE_STDLIB_H 1
#define HAVE_STRING_H 1
