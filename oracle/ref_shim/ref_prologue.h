/*
 * Prologue for the host build of the reference sources (oracle/ref_build.sh).
 * Pulls in every header the reference includes, then opens the
 * `simulation` class's private members to the harness so that H fields,
 * CPML psi arrays and the 1D incident tables can be read back for pinning.
 * TEST INFRASTRUCTURE ONLY.
 */
#pragma once
#include "cuda_runtime.h"
#include "device_launch_parameters.h"
#include <math_constants.h>
#include <iostream>
#include <math.h>
#include <mex.h>
#include <omp.h>
#include <stdint.h>
#include <stdio.h>
#define private public
