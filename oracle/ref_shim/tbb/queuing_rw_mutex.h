/* ORACLE build support: see tbb.h */
#include "tbb.h"
