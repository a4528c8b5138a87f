#include "stub_petsc.h"
