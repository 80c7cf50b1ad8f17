/* Double-precision instantiation of the CPU restatement (test infrastructure
 * only; see fea_oracle.h). */
#define R double
#define S f64
#include "fea_oracle_real.h"
