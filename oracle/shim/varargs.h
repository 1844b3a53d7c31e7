// Test infrastructure: the reference's utils.h includes the pre-standard
// <varargs.h>; the standard equivalent is <stdarg.h>.
#include <stdarg.h>
