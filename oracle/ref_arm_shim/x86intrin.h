// Empty stand-in for <x86intrin.h> (see immintrin.h in this directory).
#pragma once
#include "immintrin.h"
