/* boost::mt19937 stand-in for the oracle build: Boost's mt19937 and
 * std::mt19937 are the same MT19937 generator with the same default seed
 * (5489) and the same seeding procedure. */
#ifndef SKW_REF_SHIM_MT19937_HPP
#define SKW_REF_SHIM_MT19937_HPP
#include <random>
namespace boost {
typedef std::mt19937 mt19937;
}
#endif
