/* Minimal stand-in for the three Boost string helpers the reference's
 * physics headers name (iequals, split, is_any_of).  Oracle build only. */
#pragma once
#include <cctype>
#include <string>
#include <vector>

namespace boost {
inline bool iequals(const std::string & a, const std::string & b) {
  if(a.size() != b.size()) return false;
  for(size_t i = 0; i < a.size(); ++i)
    if(std::tolower((unsigned char)a[i]) != std::tolower((unsigned char)b[i]))
      return false;
  return true;
}
struct is_any_of_t {
  std::string set;
  bool operator()(char c) const { return set.find(c) != std::string::npos; }
};
inline is_any_of_t is_any_of(const std::string & s) { return is_any_of_t{s}; }
template<class Seq, class Pred>
Seq & split(Seq & out, const std::string & in, Pred p) {
  out.clear();
  std::string cur;
  for(char c : in) {
    if(p(c)) { out.push_back(cur); cur.clear(); }
    else cur.push_back(c);
  }
  out.push_back(cur);
  return out;
}
namespace algorithm {
using boost::iequals;
using boost::is_any_of;
using boost::split;
} // namespace algorithm
} // namespace boost
