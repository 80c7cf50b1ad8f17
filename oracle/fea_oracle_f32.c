/* Single-precision instantiation of the CPU restatement (test infrastructure
 * only; see fea_oracle.h): float is the reference's arithmetic type. */
#define R float
#define S f32
#include "fea_oracle_real.h"
