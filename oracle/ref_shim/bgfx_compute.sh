// Stand-in for bgfx's bgfx_compute.sh when the reference's compute shaders
// are compiled as C++ for the oracle: pulls in the GLSL shim types and makes
// the GLSL built-ins visible inside the namespace that wraps each shader.
#include "glsl_shim.hpp"
using namespace glsl;
