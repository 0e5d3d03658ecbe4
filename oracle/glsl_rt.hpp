// glsl_rt.hpp -- TEST INFRASTRUCTURE ONLY.
//
// The GL_EXT_ray_tracing built-ins the reference's path-tracing shaders use,
// for compiling them as C++ (with glsl_shim.hpp): the launch and hit
// variables, the ray flags, the acceleration-structure handle and
// traceRayEXT. One shader invocation runs at a time, so the built-in
// variables are plain globals that the pin driver sets before each call.
#pragma once
#include "glsl_shim.hpp"

namespace glsl {

struct accelerationStructureEXT {};

constexpr uint gl_RayFlagsOpaqueEXT = 0x01u;
constexpr uint gl_RayFlagsTerminateOnFirstHitEXT = 0x04u;
constexpr uint gl_RayFlagsSkipClosestHitShaderEXT = 0x08u;

inline uvec3 gl_LaunchIDEXT, gl_LaunchSizeEXT;
inline vec3 gl_WorldRayOriginEXT, gl_WorldRayDirectionEXT, gl_ObjectRayOriginEXT, gl_ObjectRayDirectionEXT;
inline float gl_HitTEXT;
inline int gl_InstanceCustomIndexEXT, gl_PrimitiveID;
inline mat4x3 gl_ObjectToWorldEXT;

// ignoreIntersectionEXT (an any-hit shader's jump statement): the pin driver
// reads the flag after the any-hit shader returns.
inline bool gl_IgnoreIntersection = false;

// Defined by the pin driver: traverses the oracle's BVH and runs the
// closest-hit or miss shader on the caller's payload (location 0).
void traceRayEXT(const accelerationStructureEXT& as, uint flags, uint mask, uint sbt_offset, uint sbt_stride,
                 uint miss_index, vec3 origin, float tmin, vec3 direction, float tmax, int payload);

}  // namespace glsl

// GLSL declaration qualifiers, while the shader text is compiled: interface
// blocks become structs, resource and payload qualifiers vanish.
#define layout(...)
#define uniform struct
#define readonly
#define buffer struct
#define rayPayloadEXT
#define rayPayloadInEXT
#define hitAttributeEXT
#define ignoreIntersectionEXT          \
    {                                  \
        glsl::gl_IgnoreIntersection = true; \
        return;                        \
    }
