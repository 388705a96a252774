// stand-in for the CUDA runtime header in the CPU build of the reference (see emul.h)
#pragma once
#include "../emul.h"
