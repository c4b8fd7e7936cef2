/* Declaration-only stand-in (see opencv2/core/core.hpp in this folder). */
#pragma once
#include "../core/core.hpp"
