/* Stand-in for the cachesize.h that WDutils' build generates with
 * utils/make_cachesize (getconf LEVEL1_DCACHE_LINESIZE): the L1 data-cache
 * line of the x86-64 build host and of the Arm (Neoverse V2) GPU host alike. */
#ifndef WDutils_included_cachesize_h
#define WDutils_included_cachesize_h
#include <cstddef>
namespace WDutils {
#define LEVEL1_DCACHE_LINESIZE 64
  static const std::size_t sizeof_cache_line = LEVEL1_DCACHE_LINESIZE;
}
#endif
