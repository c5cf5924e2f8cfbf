/* Reference include path of the SNNCuda C ABI (include/snncuda/c/SNNCudaC.h
 * in the reference): snncuda_version and snncuda_cuda_available, here with
 * the rest of the GB300 backend's C ABI. */
#ifndef SNNCUDA_C_SNNCUDAC_H
#define SNNCUDA_C_SNNCUDAC_H

#include "../../snncuda_gb300.h"

#endif
