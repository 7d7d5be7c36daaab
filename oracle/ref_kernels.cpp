// The reference's own compute shaders, compiled unchanged as C++ through the
// GLSL shim in ref_shim/, with a CPU dispatcher per shader.  Built only where
// the reference sources are present (oracle/build_ref.sh) into oracle/_ref/.
//
// Each shader is wrapped in its own namespace; its `uniform` and buffer
// declarations become namespace statics that the extern "C" entry points set
// before dispatching main() over a (ceil(W/16), ceil(H/16)) grid of 16x16
// invocations, in the order bgfx would number them.  Buffers use the
// reference's layouts: velocity, pressure and obstacles are vec2 per cell,
// divergence / vorticity / particles are float per cell.
//
// Test infrastructure only: used by tests/golden/make_golden.py and the CPU
// tests to pin oracle/oracle.c; never linked into the product.
#include "glsl_shim.hpp"

glsl::uvec3 gl_GlobalInvocationID;

template <class F>
static void dispatch(unsigned groups_x, unsigned groups_y, F body) {
    for (unsigned gy = 0; gy < groups_y; ++gy)
        for (unsigned gx = 0; gx < groups_x; ++gx)
            for (unsigned ty = 0; ty < 16; ++ty)
                for (unsigned tx = 0; tx < 16; ++tx) {
                    gl_GlobalInvocationID.x = gx * 16 + tx;
                    gl_GlobalInvocationID.y = gy * 16 + ty;
                    gl_GlobalInvocationID.z = 0;
                    gl_GlobalInvocationID.xy.x = gl_GlobalInvocationID.x;
                    gl_GlobalInvocationID.xy.y = gl_GlobalInvocationID.y;
                    body();
                }
}

static unsigned groups(int n) { return (unsigned)((n + 15) / 16); }

#undef COMMON_SH_HEADER_GUARD
namespace ref_ClearBuffer {
#include "shader.ClearBuffer.comp"
}
#undef COMMON_SH_HEADER_GUARD
namespace ref_InitBoundaries {
#include "shader.InitBoundaries.comp"
}
#undef COMMON_SH_HEADER_GUARD
namespace ref_AddVelocity {
#include "shader.AddVelocity.comp"
}
#undef COMMON_SH_HEADER_GUARD
namespace ref_AdvectVelocity {
#include "shader.AdvectVelocity.comp"
}
#undef COMMON_SH_HEADER_GUARD
namespace ref_CalcVorticity {
#include "shader.CalcVorticity.comp"
}
#undef COMMON_SH_HEADER_GUARD
namespace ref_ApplyVorticity {
#include "shader.ApplyVorticity.comp"
}
#undef COMMON_SH_HEADER_GUARD
namespace ref_Viscosity {
#include "shader.Viscosity.comp"
}
#undef COMMON_SH_HEADER_GUARD
namespace ref_Divergence {
#include "shader.Divergence.comp"
}
#undef COMMON_SH_HEADER_GUARD
namespace ref_Poisson {
#include "shader.Poisson.comp"
}
#undef COMMON_SH_HEADER_GUARD
namespace ref_SubtractGradient {
#include "shader.SubtractGradient.comp"
}
#undef COMMON_SH_HEADER_GUARD
namespace ref_AddCircleObstacle {
#include "shader.AddCircleObstacle.comp"
}
#undef COMMON_SH_HEADER_GUARD
namespace ref_AddTriangleObstacle {
#include "shader.AddTriangleObstacle.comp"
}
namespace ref_AddParticle {
#include "shader.AddParticle.comp"
}
namespace ref_AdvectParticle {
#include "shader.AdvectParticle.comp"
}

using glsl::vec2;

#define AS_VEC2(p) reinterpret_cast<vec2*>(p)

extern "C" {

// ClearBuffer (shader.ClearBuffer.comp): vec2 buffer -> 0 broadcast.
void ref_clear_buffer(float* buf, int W, int H) {
    using namespace ref_ClearBuffer;
    _Size = vec2((float)W, (float)H);
    _Buffer.p = AS_VEC2(buf);
    dispatch(groups(W), groups(H), [] { main(); });
}

// InitBoundaries (shader.InitBoundaries.comp): zero the border, in place.
void ref_init_boundaries(float* vel, int W, int H) {
    using namespace ref_InitBoundaries;
    _Size = vec2((float)W, (float)H);
    _VelocityIn.p = AS_VEC2(vel);
    dispatch(groups(W), groups(H), [] { main(); });
}

// AddVelocity (shader.AddVelocity.comp).
void ref_add_velocity(const float* vin, float* vout, int W, int H, float px, float py,
                      float vx, float vy, float radius) {
    using namespace ref_AddVelocity;
    _Size = vec2((float)W, (float)H);
    _VelocityIn.p = AS_VEC2(const_cast<float*>(vin));
    _VelocityOut.p = AS_VEC2(vout);
    _Position = vec2(px, py);
    _Value = vec2(vx, vy);
    _Radius = radius;
    dispatch(groups(W), groups(H), [] { main(); });
}

// AdvectVelocity (shader.AdvectVelocity.comp).
void ref_advect_velocity(const float* vin, float* vout, const float* obs, int W, int H,
                         float dt, float speed, float dissipation) {
    using namespace ref_AdvectVelocity;
    _Size = vec2((float)W, (float)H);
    _VelocityIn.p = AS_VEC2(const_cast<float*>(vin));
    _VelocityOut.p = AS_VEC2(vout);
    _Obstacles.p = AS_VEC2(const_cast<float*>(obs));
    _ElapsedTime = dt;
    _Speed = speed;
    _Dissipation = dissipation;
    dispatch(groups(W), groups(H), [] { main(); });
}

// CalcVorticity (shader.CalcVorticity.comp).
void ref_calc_vorticity(const float* vin, float* vort, int W, int H) {
    using namespace ref_CalcVorticity;
    _Size = vec2((float)W, (float)H);
    _VelocityIn.p = AS_VEC2(const_cast<float*>(vin));
    _Vorticity.p = vort;
    dispatch(groups(W), groups(H), [] { main(); });
}

// ApplyVorticity (shader.ApplyVorticity.comp).
void ref_apply_vorticity(const float* vin, float* vout, const float* vort, int W, int H,
                         float dt, float scale) {
    using namespace ref_ApplyVorticity;
    _Size = vec2((float)W, (float)H);
    _VelocityIn.p = AS_VEC2(const_cast<float*>(vin));
    _VelocityOut.p = AS_VEC2(vout);
    _Vorticity.p = const_cast<float*>(vort);
    _ElapsedTime = dt;
    _VorticityScale = scale;
    dispatch(groups(W), groups(H), [] { main(); });
}

// Viscosity (shader.Viscosity.comp).
void ref_viscosity(const float* vin, float* vout, int W, int H, float alpha, float rbeta) {
    using namespace ref_Viscosity;
    _Size = vec2((float)W, (float)H);
    _VelocityIn.p = AS_VEC2(const_cast<float*>(vin));
    _VelocityOut.p = AS_VEC2(vout);
    _Alpha = alpha;
    _rBeta = rbeta;
    dispatch(groups(W), groups(H), [] { main(); });
}

// Divergence (shader.Divergence.comp).
void ref_divergence(const float* vin, const float* obs, float* div, int W, int H) {
    using namespace ref_Divergence;
    _Size = vec2((float)W, (float)H);
    _VelocityIn.p = AS_VEC2(const_cast<float*>(vin));
    _Obstacles.p = AS_VEC2(const_cast<float*>(obs));
    _Divergence.p = div;
    dispatch(groups(W), groups(H), [] { main(); });
}

// Poisson (shader.Poisson.comp): one Jacobi sweep, pressure as vec2 per cell.
void ref_poisson(const float* pin, float* pout, const float* div, const float* obs, int W,
                 int H) {
    using namespace ref_Poisson;
    _Size = vec2((float)W, (float)H);
    _PressureIn.p = AS_VEC2(const_cast<float*>(pin));
    _PressureOut.p = AS_VEC2(pout);
    _Divergence.p = const_cast<float*>(div);
    _Obstacles.p = AS_VEC2(const_cast<float*>(obs));
    dispatch(groups(W), groups(H), [] { main(); });
}

// SubtractGradient (shader.SubtractGradient.comp).
void ref_subtract_gradient(const float* vin, float* vout, const float* p, const float* obs,
                           int W, int H) {
    using namespace ref_SubtractGradient;
    _Size = vec2((float)W, (float)H);
    _VelocityIn.p = AS_VEC2(const_cast<float*>(vin));
    _VelocityOut.p = AS_VEC2(vout);
    _PressureIn.p = AS_VEC2(const_cast<float*>(p));
    _Obstacles.p = AS_VEC2(const_cast<float*>(obs));
    dispatch(groups(W), groups(H), [] { main(); });
}

// AddCircleObstacle (shader.AddCircleObstacle.comp).
void ref_add_circle_obstacle(float* obs, int W, int H, float px, float py, float radius,
                             int is_static) {
    using namespace ref_AddCircleObstacle;
    _Size = vec2((float)W, (float)H);
    _Obstacles.p = AS_VEC2(obs);
    _Position = vec2(px, py);
    _Radius = radius;
    _Static = is_static ? 1.0f : 0.0f;
    dispatch(groups(W), groups(H), [] { main(); });
}

// AddTriangleObstacle (shader.AddTriangleObstacle.comp).
void ref_add_triangle_obstacle(float* obs, int W, int H, float x1, float y1, float x2,
                               float y2, float x3, float y3, int is_static) {
    using namespace ref_AddTriangleObstacle;
    _Size = vec2((float)W, (float)H);
    _Obstacles.p = AS_VEC2(obs);
    _P1 = vec2(x1, y1);
    _P2 = vec2(x2, y2);
    _P3 = vec2(x3, y3);
    _Static = is_static ? 1.0f : 0.0f;
    dispatch(groups(W), groups(H), [] { main(); });
}

// AddParticle (demo/shaders/shader.AddParticle.comp).  The reference dispatches
// it with the x group count in both dimensions (demo/smooth_particles_area.py:80-81);
// `groups_y_override` > 0 reproduces that dispatch shape.
void ref_add_particle(const float* rin, float* rout, int Wp, int Hp, float px, float py,
                      float radius, float value, int groups_y_override) {
    using namespace ref_AddParticle;
    _ParticleSize = vec2((float)Wp, (float)Hp);
    _ParticlesIn.p = const_cast<float*>(rin);
    _ParticlesOut.p = rout;
    _Position = vec2(px, py);
    _Radius = radius;
    _Value = value;
    unsigned gy = groups_y_override > 0 ? (unsigned)groups_y_override : groups(Hp);
    dispatch(groups(Wp), gy, [] { main(); });
}

// AdvectParticle (demo/shaders/shader.AdvectParticle.comp).
void ref_advect_particle(const float* rin, float* rout, const float* vel, const float* obs,
                         int Wp, int Hp, int Wv, int Hv, float dt, float speed,
                         float dissipation) {
    using namespace ref_AdvectParticle;
    _ParticleSize = vec2((float)Wp, (float)Hp);
    _VelocitySize = vec2((float)Wv, (float)Hv);
    _ParticlesIn.p = const_cast<float*>(rin);
    _ParticlesOut.p = rout;
    _Velocity.p = AS_VEC2(const_cast<float*>(vel));
    _Obstacles.p = AS_VEC2(const_cast<float*>(obs));
    _ElapsedTime = dt;
    _Speed = speed;
    _Dissipation = dissipation;
    dispatch(groups(Wp), groups(Hp), [] { main(); });
}

}  // extern "C"
