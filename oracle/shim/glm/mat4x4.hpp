// Oracle test infrastructure: forwards to the glm-compatible shim.
#pragma once
#include "glm_shim.hpp"
