/* Stand-in for the CUDA samples' helper_functions.h, which the reference's
 * cu_device.h includes and this machine does not have.  The reference code
 * compiled by oracle/ref uses only the C library from it.  TEST
 * INFRASTRUCTURE ONLY. */
#pragma once
#include <cmath>
#include <cstdio>
#include <cstdlib>
