// Minimal stand-in for sdsl-lite's bit_vectors.hpp (TEST INFRASTRUCTURE ONLY;
// see int_vector.hpp in this directory): bit_vector with the rank and select
// support headers.
#ifndef WTG_SDSL_SHIM_BIT_VECTORS
#define WTG_SDSL_SHIM_BIT_VECTORS
#include "int_vector.hpp"
#include "rank_support.hpp"
#include "select_support.hpp"
#endif
