/* The reference only names boost::multiprecision::uint128_t in a using
 * declaration (tree.h); the hot path keys are uint64_t.  Oracle build only. */
#pragma once
namespace boost {
namespace multiprecision {
typedef unsigned __int128 uint128_t;
} // namespace multiprecision
} // namespace boost
