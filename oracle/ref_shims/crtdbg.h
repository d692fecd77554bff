/* Stand-in for the MSVC debug CRT header used by the reference's ASSERT
 * macro (oracle build only). */
#ifndef SKW_REF_SHIM_CRTDBG_H
#define SKW_REF_SHIM_CRTDBG_H
#include <cassert>
#include <cmath>
#define _ASSERTE(expr) assert(expr)
#define _isnan(x) std::isnan(x)
#define _finite(x) std::isfinite(x)
#endif
