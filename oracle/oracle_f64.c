/* Double instantiation of the oracle (TEST INFRASTRUCTURE ONLY): the FP64 re-run of every step. */
#define R double
#define R_IS_DOUBLE 1
#define P ord_
#include "oracle.h"
#include "oracle_impl.h"
