/* Test-only stub for the two Boost string helpers the reference's RRNG
 * reader uses: split(tokens, line, is_any_of(" \t")).  Semantics follow
 * Boost's documented default (token_compress_off): every delimiter ends a
 * token, so consecutive delimiters yield empty tokens. */
#ifndef PP_ORACLE_STUB_BOOST_STRING_HPP
#define PP_ORACLE_STUB_BOOST_STRING_HPP
#include <string>
#include <vector>
namespace boost {
struct pp_any_of { std::string set; };
inline pp_any_of is_any_of(const char* s) { return pp_any_of{std::string(s)}; }
inline std::vector<std::string>& split(std::vector<std::string>& out,
                                       const std::string& in, const pp_any_of& d) {
  out.clear();
  std::string cur;
  for (char c : in) {
    if (d.set.find(c) != std::string::npos) { out.push_back(cur); cur.clear(); }
    else cur.push_back(c);
  }
  out.push_back(cur);
  return out;
}
}  // namespace boost
#endif
