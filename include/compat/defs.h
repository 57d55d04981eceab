/* defs.h -- stands in for the reference header utils/defs.h: every declaration it makes
 * (prototypes, result structs, option structs and helpers) is in corrfunc_gb300.h, so
 * programs written against the reference build unchanged with -I include/compat. */
#pragma once
#include "../corrfunc_gb300.h"
