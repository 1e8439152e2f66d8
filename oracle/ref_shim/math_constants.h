/* Host-only stand-in (see cuda_runtime.h). */
#pragma once
#define CUDART_PI_F 3.141592654f
