// Minimal stand-in for sdsl-lite's wt_helper.hpp and the iterator / buffer
// names wt_int's declarations mention (TEST INFRASTRUCTURE ONLY; see
// int_vector.hpp in this directory).  Only the names, the range types and
// the raw-bytes member I/O are restated: a range is a closed interval
// [first, second] of positions.
#ifndef WTG_SDSL_SHIM_WT_HELPER
#define WTG_SDSL_SHIM_WT_HELPER
#include <cstdint>
#include <string>
#include <utility>
#include <vector>
#include "int_vector.hpp"

namespace sdsl {
typedef std::pair<uint64_t, uint64_t> range_type;
typedef std::vector<range_type> range_vec_type;

template <class t_rac>
class random_access_const_iterator {
 public:
  random_access_const_iterator(const t_rac*, uint64_t) {}
};

template <uint8_t t_width = 0>
class int_vector_buffer {
 public:
  uint64_t size() const { return 0; }
  uint8_t width() const { return 64; }
  std::string filename() const { return std::string(); }
  uint64_t operator[](uint64_t) const { return 0; }
};

inline std::string tmp_file(const std::string& f, const std::string& s) { return f + s; }
inline int remove(const std::string&) { return 0; }
template <class T>
bool load_from_file(T&, const std::string&) { return false; }
// write_member / read_member of a plain value: its sizeof(T) bytes as they
// lie in memory
template <class T>
uint64_t write_member(const T& t, std::ostream& out, structure_tree_node* = nullptr, std::string = "") {
  out.write(reinterpret_cast<const char*>(&t), sizeof(T));
  return sizeof(T);
}
template <class T>
void read_member(T& t, std::istream& in) {
  in.read(reinterpret_cast<char*>(&t), sizeof(T));
}
}  // namespace sdsl
#endif
