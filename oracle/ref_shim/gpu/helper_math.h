// stand-in: see ref_gpu_shim.h
#pragma once
#include "ref_gpu_shim.h"
