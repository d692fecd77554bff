/* Force-included ahead of every reference translation unit in the oracle
 * build: the reference was written against MSVC, whose headers pull these
 * in transitively. */
#ifndef SKW_REF_SHIM_PRELUDE_H
#define SKW_REF_SHIM_PRELUDE_H
#include <climits>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <cstdlib>
#include <algorithm>
#include <limits>
#include <string>
#include <vector>
#include <utility>
#include <memory>
#include <numeric>
#include <queue>
#include "windows.h"
#endif
