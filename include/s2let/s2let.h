/*
 * s2let.h: the umbrella header of the S2LET C API (include/s2let/s2let.h of
 * S2LET 2.2.7), so that a caller's `#include <s2let.h>` (with -I<prefix>/include/s2let)
 * or `#include <s2let/s2let.h>` (with -I<prefix>/include) builds unchanged
 * against libs2let_gpu.so.  It includes the per-module headers below, which
 * forward to s2let_gpu.h.  Not provided, because libs2let_gpu.so does not
 * implement them: the HEALPix, IDL and MATLAB glue (s2let_hpx.h,
 * s2let_idl_*.h, s2let_transform_axisym_hpx.h, s2let_mex.h), the demo headers
 * and the random-flm test helpers of s2let_lm.h.
 */
#ifndef S2LET
#define S2LET
#include "s2let_alloc.h"
#include "s2let_analysis.h"
#include "s2let_analysis_adjoint.h"
#include "s2let_error.h"
#include "s2let_fits.h"
#include "s2let_helper.h"
#include "s2let_lm.h"
#include "s2let_math.h"
#include "s2let_mw.h"
#include "s2let_so3.h"
#include "s2let_synthesis.h"
#include "s2let_synthesis_adjoint.h"
#include "s2let_tiling.h"
#include "s2let_transform_axisym_lm.h"
#include "s2let_transform_axisym_mw.h"
#include "s2let_types.h"
#endif
