// Internal header of the host-side sources (file formats, synthetic problems).
#pragma once
#include "plsqr_gpu.h"
