/* Include shim: the network factory only names glm::vec3/uvec3 in
 * declarations it inherits from morphology.h. */
#pragma once
namespace glm {
struct vec3 { float x, y, z; };
struct uvec3 { unsigned x, y, z; };
}  // namespace glm
