// Declarations shared by the setup kernels (epr_setup.cu) and the C ABI.
#pragma once
#include "epr_context.h"
