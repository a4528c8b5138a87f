#ifndef P4_TO_P8
#define P4_TO_P8 1
#endif
#include "stub_core.h"
