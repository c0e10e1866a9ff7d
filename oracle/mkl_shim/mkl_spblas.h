/* Stand-in: see mkl.h in this folder. */
#include "mkl.h"
