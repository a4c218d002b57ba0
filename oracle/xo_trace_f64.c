/* Oracle (test infrastructure only): FP64 instantiation of the shader
 * restatement -- the per-ray emission re-trace. */
#define XO_REAL double
#define XO_ENTRY xo_render_f64
#include "xo_trace_impl.h"
