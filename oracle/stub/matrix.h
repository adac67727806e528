/* Empty stand-in for MATLAB's matrix.h; everything needed is in mex.h. */
#include "mex.h"
