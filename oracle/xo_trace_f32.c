/* Oracle (test infrastructure only): FP32 instantiation of the shader
 * restatement -- the image oracle and the timed CPU baseline. */
#define XO_REAL float
#define XO_ENTRY xo_render_f32
#include "xo_trace_impl.h"
