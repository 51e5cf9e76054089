// The box pyramid of examples3d/pyramid3.rs (base 20, half extents 0.5, 1.0
// spacing, on a 50 x 1 x 50 ground), written against the C++ mirror of the
// nphysics3d world API and stepped on the GPU. Prints "<body slot> <7 pose
// floats>" per box after the requested number of steps (bit patterns in hex).
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "../../nphysics_gb300/cpp/gpu_mechanical_world.hpp"

using namespace nphysics_gpu;

int main(int argc, char** argv) {
    int steps = argc > 1 ? std::atoi(argv[1]) : 10;
    GpuMechanicalWorld mechanical_world(Vector3{0.0f, -9.81f, 0.0f}, 256, 256, 4096);
    DefaultGeometricalWorld geometrical_world;
    DefaultBodySet bodies;
    DefaultColliderSet colliders;
    DefaultJointConstraintSet joint_constraints;
    DefaultForceGeneratorSet force_generators;

    DefaultBodyHandle ground = bodies.insert(Ground{});
    colliders.insert(ColliderDesc::cuboid(Vector3{50.0f, 1.0f, 50.0f})
                         .translation(Vector3{0.0f, -1.0f, 0.0f})
                         .build(BodyPartHandle{ground, 0}));
    const int base = 20;
    for (int row = 0; row < base; ++row) {
        for (int i = 0; i < base - row; ++i) {
            float x = float(i * 1.0 + row * 0.5 - (base - 1) * 0.5);
            float y = float(0.5 + row * 1.0);
            RigidBody rb = RigidBodyDesc().translation(Vector3{x, y, 0.0f}).build();
            DefaultBodyHandle h = bodies.insert(rb);
            colliders.insert(ColliderDesc::cuboid(Vector3{0.5f, 0.5f, 0.5f}).density(1.0f).build(BodyPartHandle{h, 0}));
        }
    }
    try {
        for (int s = 0; s < steps; ++s)
            mechanical_world.step(geometrical_world, bodies, colliders, joint_constraints, force_generators);
        // A non-empty joint set is rejected, not run on the CPU.
        joint_constraints.insert_placeholder();
        try {
            mechanical_world.step(geometrical_world, bodies, colliders, joint_constraints, force_generators);
            std::printf("ERROR joints accepted\n");
            return 1;
        } catch (const Error& e) {
            if (e.status != NPGPU_ERR_NONEMPTY_JOINTS) return 1;
        }
    } catch (const Error& e) {
        std::fprintf(stderr, "step failed: %s\n", e.what());
        return 2;
    }
    for (uint64_t i = 1; i <= 210; ++i) {
        const RigidBody* rb = bodies.rigid_body(DefaultBodyHandle{i, 0});
        if (!rb) return 3;
        std::printf("%llu", (unsigned long long)i);
        for (int k = 0; k < 7; ++k) {
            uint32_t bits;
            std::memcpy(&bits, &rb->desc.position[k], 4);
            std::printf(" %08x", bits);
        }
        std::printf("\n");
    }
    return 0;
}
