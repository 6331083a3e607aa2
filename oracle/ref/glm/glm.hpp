// Minimal GLM-compatible umbrella header (see vec4.hpp, vec2.hpp).
#pragma once
#include "mat4x4.hpp"
#include "vec2.hpp"
#include "vec4.hpp"
