/* Host-only stand-in (see cuda_runtime.h). */
#pragma once
