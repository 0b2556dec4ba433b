// Stand-in for <arcane/utils/FatalErrorException.h>: ARCANE_FATAL / ARCANE_THROW.
#pragma once
#include "../ArcaneShim.h"
