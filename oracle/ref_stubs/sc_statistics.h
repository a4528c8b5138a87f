#include "stub_core.h"
