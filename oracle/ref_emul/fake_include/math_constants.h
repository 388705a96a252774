// stand-in for math_constants.h in the CPU build of the reference (no constant is used)
#pragma once
