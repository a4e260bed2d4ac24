/* Stand-in for the CUDA samples' helper_timer.h (unused by the host build).
 * TEST INFRASTRUCTURE ONLY. */
#pragma once
