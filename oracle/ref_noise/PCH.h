// PCH.h -- stands in for the reference's precompiled header (the engine
// includes); the reference's noise sources include it first.
#pragma once
#include "ez_shim.h"
