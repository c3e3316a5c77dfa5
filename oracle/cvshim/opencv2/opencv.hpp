// OpenCV header name used by the reference sources; forwards to the oracle/_ref shim.
#pragma once
#include "zim_cv.hpp"
