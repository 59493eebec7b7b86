// Minimal stand-in for sdsl-lite's sdsl_concepts.hpp (TEST INFRASTRUCTURE
// ONLY; see int_vector.hpp in this directory): the category tags wt_int and
// wt_pc name in their typedefs.
#ifndef WTG_SDSL_SHIM_CONCEPTS
#define WTG_SDSL_SHIM_CONCEPTS
namespace sdsl {
struct wt_tag {};
struct int_alphabet_tag {};
struct byte_alphabet_tag {};
}  // namespace sdsl
#endif
