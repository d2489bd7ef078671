/* CPU shim: intentionally empty so the reference sources compile as host C++. */
#pragma once
#include "cuda_runtime.h"
