/* Float instantiation of the oracle (TEST INFRASTRUCTURE ONLY): the reference's FP32 arithmetic. */
#define R float
#define R_IS_DOUBLE 0
#define P orf_
#include "oracle.h"
#include "oracle_impl.h"
