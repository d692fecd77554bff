/* boost::mt19937 stand-in for the oracle build.
 *
 * Boost's mt19937 is the MT19937 generator (default seed 5489, the standard
 * seeding procedure) with a 32-bit result_type.  std::mt19937 is the same
 * generator but declares result_type as uint_fast32_t, which is 64 bits wide
 * on LP64 Linux.  The reference's RandomGenerator scales draws by
 * 1 / (1 + numeric_limits<result_type>::max()), so the std typedef would make
 * every draw ~2^-32 (all sampler jitter and sample sequences become 0).  The
 * engine is therefore instantiated with uint32_t, as Boost's is. */
#ifndef SKW_REF_SHIM_MT19937_HPP
#define SKW_REF_SHIM_MT19937_HPP
#include <cstdint>
#include <random>
namespace boost {
typedef std::mersenne_twister_engine<uint32_t, 32, 624, 397, 31, 0x9908b0dfu, 11, 0xffffffffu, 7, 0x9d2c5680u, 15,
                                     0xefc60000u, 18, 1812433253u>
    mt19937;
}
#endif
