/* Drop-in include path: callers that #include "qkrylov/c_api.h" get the GB300
 * library's C ABI (a superset of the reference's). */
#include "../qkrylov_c_api.h"
