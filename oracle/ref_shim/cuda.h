// TEST INFRASTRUCTURE ONLY (oracle): host stand-in, see cuda_runtime.h.
#pragma once
#include "cuda_runtime.h"
