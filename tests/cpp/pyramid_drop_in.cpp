// The box pyramid of examples3d/pyramid3.rs (base 20, half extents 0.5, 1.0
// spacing, on a 50 x 1 x 50 ground), written against the C++ mirror of the
// nphysics3d world API and stepped on the GPU. Prints "<body slot> <7 pose
// floats>" per box after the requested number of steps (bit patterns in hex),
// then checks a ball-jointed pendulum in a second world.
#include <cmath>
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
        // A pendulum in a world of its own: a ball on a 2 m ball joint from a
        // pivot on the ground, released at 0.1 rad, keeps its rod length,
        // and its joint carries about m g dt when it passes the bottom.
        GpuMechanicalWorld pendulum_world(Vector3{0.0f, -9.81f, 0.0f}, 16, 16, 1024);
        DefaultBodySet pb;
        DefaultColliderSet pc;
        DefaultJointConstraintSet pj;
        DefaultBodyHandle pg = pb.insert(Ground{});
        const float len = 2.0f, a = 0.1f;
        RigidBody ball = RigidBodyDesc().translation(Vector3{len * std::sin(a), 10.0f - len * std::cos(a), 0.0f}).build();
        DefaultBodyHandle bh = pb.insert(ball);
        pc.insert(ColliderDesc::ball(0.1f).density(100.0f).build(BodyPartHandle{bh, 0}));
        DefaultJointConstraintHandle jh = pj.insert(BallConstraint(BodyPartHandle{pg, 0}, BodyPartHandle{bh, 0},
                                                                   Vector3{0.0f, 10.0f, 0.0f},
                                                                   Vector3{-len * std::sin(a), len * std::cos(a), 0.0f}));
        for (int s = 0; s < 60; ++s)
            pendulum_world.step(geometrical_world, pb, pc, pj, force_generators);
        const RigidBody* prb = pb.rigid_body(bh);
        const float dx = prb->desc.position[0], dy = prb->desc.position[1] - 10.0f;
        const float rod = std::sqrt(dx * dx + dy * dy);
        const BallConstraint& bc = std::get<BallConstraint>(*pj.get(jh));
        if (std::fabs(rod - len) > 4e-3f || bc.is_broken() || !(std::fabs(bc.impulses()[1]) > 0.05f)) {
            std::fprintf(stderr, "pendulum: rod %f impulse %f\n", rod, bc.impulses()[1]);
            return 4;
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
