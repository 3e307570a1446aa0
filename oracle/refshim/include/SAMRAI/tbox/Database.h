#include "SAMRAI/shim_core.h"
