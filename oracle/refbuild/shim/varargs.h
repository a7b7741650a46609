/* varargs.h mapped to stdarg.h for the oracle build */
#include <stdarg.h>
