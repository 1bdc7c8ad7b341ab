// Stand-in for the CUDA header of this name (oracle/ref_emu): everything lives in emu.h.
#pragma once
#include "emu.h"
