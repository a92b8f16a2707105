// Oracle test infrastructure: stands in for the reference's ECS/ECStypes.h
// (inMyRoom_vulkan/include/ECS/ECStypes.h), which pulls in glm quaternions and
// Vulkan shader headers. It declares only the collision boundary types with the
// reference's field order (ECStypes.h:18, 149-163) so that the reference's
// collision translation units compile unchanged against the glm shim.
#pragma once

#include <cstdint>
#include <map>
#include <memory>
#include <set>
#include <string>
#include <unordered_map>  // the real header's standard includes (ECStypes.h:3-8), which
#include <vector>         // the reference's translation units rely on

#include "glm/mat4x4.hpp"
#include "glm/vec3.hpp"

typedef uint16_t Entity;

struct CollisionDetectionEntry
{
    glm::mat4x4 currentGlobalMatrix;
    glm::mat4x4 previousGlobalMatrix;
    const class OBBtree* OBBtree_ptr;
    bool shouldCallback;
    Entity entity;
};

struct CollisionCallbackData
{
    Entity familyEntity;
    Entity collideWithEntity;
    glm::vec3 deltaVector = glm::vec3(0.f, 0.f, 0.f);
};
