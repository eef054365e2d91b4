// GpuWorld.hpp -- a world type for PlayRho's type-erased World whose Step runs
// on the GPU through include/prgpu.h:
//
//     playrho::d2::World world{playrho::d2::GpuWorld{}};
//     // ... CreateBody / CreateShape / Attach / CreateJoint as with any World ...
//     const auto stats = Step(world, stepConf);   // the GB300 world step
//
// World's templated constructor (Library/include/playrho/d2/World.hpp:739-745)
// wraps any type for which detail::WorldModel<T> (detail/WorldModel.hpp:36-374)
// finds the free functions declared below by argument-dependent lookup; they are
// the set WorldConcept (detail/WorldConcept.hpp:66-407) requires, with the
// signatures of their AabbTreeWorld counterparts (AabbTreeWorld.hpp:120-531).
// Everything above -- the World free functions in World*.hpp and their sources
// -- works unchanged, so a program switches by changing the constructor call.
//
// What the GPU world does differently, by design of this path:
//  * disk, polygon, edge, chain and multi shapes; a chain's edges and a multi
//    shape's hulls are shapes of the GPU batch, one proxy per child as in the
//    reference; StepConf::doToi runs the time-of-impact phase, with sub-stepping
//    (one event per Step, IsStepComplete) as the reference offers it; a world
//    rebuilt while its step is incomplete starts complete;
//  * Gauss-Seidel sweeps visit contacts in colour order, not island order;
//  * contact IDs are the GPU's contact slots: stable for a contact's life and
//    reused after it is destroyed, as the reference's pools reuse them;
//    SetContact (enabled, friction, restitution, tangent speed) and SetManifold
//    take effect from the next step;
//  * the contact listeners are called from Step after the GPU step, phase by
//    phase in the order the reference calls them (EndContact of the touching
//    contacts the step destroyed; BeginContact / EndContact / PreSolveContact of
//    the contacts the pre-phase updated; PostSolveContact of the solved
//    contacts; then those of the post-solve and time-of-impact updates), each
//    phase in contact-list order; while they run the world is locked.  Within
//    the post-solve calls the order is contact-list order, not island order;
//    the time-of-impact phase's own PostSolveContact calls are not made, and
//    its PreSolveContact calls pass the manifold after the step;
//  * changing anything but a body's position or velocity between steps
//    (creating or destroying entities, attaching shapes, changing a body's type,
//    flags or mass) rebuilds the GPU batch: contacts are found again on the next
//    step and start without warm-start impulses.
// Needs the PlayRho headers and library; the GPU side is libprgpu_host.so.
#pragma once

#include <optional>
#include <vector>

#include "playrho/d2/Body.hpp"
#include "playrho/d2/BodyConf.hpp"
#include "playrho/d2/DynamicTree.hpp"
#include "playrho/d2/Joint.hpp"
#include "playrho/d2/Manifold.hpp"
#include "playrho/d2/Shape.hpp"
#include "playrho/d2/WorldConf.hpp"
#include "playrho/BodyShapeFunction.hpp"
#include "playrho/Contact.hpp"
#include "playrho/ContactFunction.hpp"
#include "playrho/d2/ContactImpulsesFunction.hpp"
#include "playrho/d2/ContactManifoldFunction.hpp"
#include "playrho/JointFunction.hpp"
#include "playrho/KeyedContactID.hpp"
#include "playrho/ShapeFunction.hpp"
#include "playrho/StepConf.hpp"
#include "playrho/StepStats.hpp"
#include "playrho/pmr/StatsResource.hpp"

#include "host_world.hpp"

namespace playrho::d2 {

class GpuWorld {
public:
    explicit GpuWorld(const WorldConf& conf = WorldConf{}, int device = 0);

    // state shared with the free functions below
    WorldConf conf;
    prgpu::HostWorld host;
    std::vector<Body> bodies;    // by BodyID; the GPU's positions and velocities after each step
    std::vector<Shape> shapes;   // by ShapeID
    std::vector<Joint> joints;   // by JointID
    ShapeFunction shapeDestructionListener;
    BodyShapeFunction detachListener;
    JointFunction jointDestructionListener;
    ContactFunction beginContactListener, endContactListener;
    ContactManifoldFunction preSolveContactListener;
    ContactImpulsesFunction postSolveContactListener;
    Frequency invDeltaTime{};
    bool subStepping = false;
    bool locked = false;
    // caches rebuilt after each step, on first use
    mutable bool contactsValid = false;
    mutable std::vector<KeyedContactID> keyedContacts;  // live contacts in ContactKey order
    mutable std::vector<Contact> contacts;               // by position in keyedContacts
    mutable std::vector<Manifold> manifolds;
    mutable std::vector<uint64_t> contactSeq;            // creation number of each (contact-list order)
    mutable std::vector<int32_t> contactIndex;           // ContactID (slot) -> position, or -1
    // contacts after the last step (for the listener calls of the next), by creation number
    struct Snapshot {
        uint64_t seq;
        bool touching;
        Contact contact;
        Manifold manifold;
    };
    std::vector<std::pair<uint32_t, Snapshot>> previous;
    bool listening = false;  // `previous` holds the contacts after the last step
    const std::vector<std::pair<uint32_t, Snapshot>>* replaying = nullptr;  // while listeners run
    mutable bool treeValid = false;
    mutable DynamicTree tree;

    void Invalidate() noexcept { contactsValid = false; treeValid = false; }
    void Refresh() const;  // contacts and manifolds from the GPU
};

void SetShapeDestructionListener(GpuWorld& world, ShapeFunction listener) noexcept;
void SetDetachListener(GpuWorld& world, BodyShapeFunction listener) noexcept;
void SetJointDestructionListener(GpuWorld& world, JointFunction listener) noexcept;
void SetBeginContactListener(GpuWorld& world, ContactFunction listener) noexcept;
void SetEndContactListener(GpuWorld& world, ContactFunction listener) noexcept;
void SetPreSolveContactListener(GpuWorld& world, ContactManifoldFunction listener) noexcept;
void SetPostSolveContactListener(GpuWorld& world, ContactImpulsesFunction listener) noexcept;

bool operator==(const GpuWorld& lhs, const GpuWorld& rhs) noexcept;
std::optional<pmr::StatsResource::Stats> GetResourceStats(const GpuWorld& world) noexcept;
void Clear(GpuWorld& world) noexcept;
StepStats Step(GpuWorld& world, const StepConf& conf);
bool IsStepComplete(const GpuWorld& world) noexcept;
bool GetSubStepping(const GpuWorld& world) noexcept;
void SetSubStepping(GpuWorld& world, bool flag) noexcept;
const DynamicTree& GetTree(const GpuWorld& world) noexcept;
bool IsLocked(const GpuWorld& world) noexcept;
void ShiftOrigin(GpuWorld& world, const Length2& newOrigin);
Interval<Positive<Length>> GetVertexRadiusInterval(const GpuWorld& world) noexcept;
Frequency GetInvDeltaTime(const GpuWorld& world) noexcept;

BodyCounter GetBodyRange(const GpuWorld& world) noexcept;
std::vector<BodyID> GetBodies(const GpuWorld& world);
std::vector<BodyID> GetBodiesForProxies(const GpuWorld& world);
BodyID CreateBody(GpuWorld& world, const Body& body);
Body GetBody(const GpuWorld& world, BodyID id);
void SetBody(GpuWorld& world, BodyID id, const Body& value);
void Destroy(GpuWorld& world, BodyID id);
std::vector<std::pair<BodyID, JointID>> GetJoints(const GpuWorld& world, BodyID id);
std::vector<std::tuple<ContactKey, ContactID>> GetContacts(const GpuWorld& world, BodyID id);
std::vector<ShapeID> GetShapes(const GpuWorld& world, BodyID id);

JointCounter GetJointRange(const GpuWorld& world) noexcept;
std::vector<JointID> GetJoints(const GpuWorld& world);
JointID CreateJoint(GpuWorld& world, const Joint& def);
Joint GetJoint(const GpuWorld& world, JointID id);
void SetJoint(GpuWorld& world, JointID id, const Joint& def);
void Destroy(GpuWorld& world, JointID id);

ShapeCounter GetShapeRange(const GpuWorld& world) noexcept;
ShapeID CreateShape(GpuWorld& world, const Shape& def);
Shape GetShape(const GpuWorld& world, ShapeID id);
void SetShape(GpuWorld& world, ShapeID id, const Shape& def);
void Destroy(GpuWorld& world, ShapeID id);

ContactCounter GetContactRange(const GpuWorld& world) noexcept;
std::vector<KeyedContactID> GetContacts(const GpuWorld& world);
Contact GetContact(const GpuWorld& world, ContactID id);
void SetContact(GpuWorld& world, ContactID id, const Contact& value);
Manifold GetManifold(const GpuWorld& world, ContactID id);
void SetManifold(GpuWorld& world, ContactID id, const Manifold& value);

}  // namespace playrho::d2
