// Stand-in for Velvet/Common.hpp when the reference's solver sources are compiled on the
// CPU with g++ — TEST INFRASTRUCTURE.  The real header does not compile with g++: its
// VtCallback::Invoke re-declares the class's template parameter pack TArgs, which MSVC
// accepts and g++ rejects, and its parameter block pulls in imgui for the GUI.  The
// kernels need only the two types below: VtSimParams with the field list, types and
// order of Velvet/Common.hpp:19-48 (the emulation driver sets every field explicitly, so
// no default value is taken from here; the defaults are checked against the real header's
// text by the tests) and ColliderType (Velvet/Common.hpp:113-118).
#pragma once

#include <glm/glm.hpp>

struct VtSimParams {
    int numSubsteps;
    int numIterations;
    int maxNumNeighbors;
    float maxSpeed;
    glm::vec3 gravity;
    float bendCompliance;
    float damping;
    float relaxationFactor;
    float longRangeStretchiness;
    float collisionMargin;
    float friction;
    bool enableSelfCollision;
    int interleavedHash;
    unsigned int numParticles;
    float particleDiameter;
    float deltaTime;
    float particleDiameterScalar;
    float hashCellSizeScalar;
};

enum class ColliderType {
    Sphere,
    Plane,
    Cube,
};
