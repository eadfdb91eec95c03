// The particle classes live in particle.h (one header on the GB300 path).
#pragma once
#include "particle.h"
