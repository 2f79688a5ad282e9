/*
 * cpgpu.h — C ABI of the GB300 per-step contact path of the ConstraintPhysics
 * rigid-body engine.
 *
 * The reference engine has no FFI: its operator API is the C++ class
 * phyz::PhysicsEngine (ConstraintPhysics/src/PhysicsEngine.h:60-161).  Every
 * entry point below replaces one member of that class (or one RigidBody
 * setter) and is cited beside its declaration.  Conventions:
 *   - every function returns an int status (CPGPU_OK == 0, negative on error);
 *     no C++ exception crosses this boundary (the reference uses assert only);
 *   - all arguments are plain pointers, sizes and doubles (the reference is
 *     FP64 at its API; the device path computes in FP32);
 *   - body ids start at 1 and increase by one per created body, exactly like
 *     PhysicsEngine::next_id (PhysicsEngine.h:172, PhysicsEngine.cpp:487);
 *   - vectors are xyz triples, quaternions are (r, i, j, k) as in
 *     mthz::Quaternion (Math/src/Quaternion.h:8).
 *
 * The same function set (with prefix cpref_ for the reference engine itself
 * and cport_ for the CPU restatement) is exported by the oracle libraries under
 * oracle/, so one test harness drives all three.
 */
#ifndef CPGPU_H
#define CPGPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define CPGPU_OK                 0
#define CPGPU_ERR_INVALID_ARG   -1  /* bad handle, id, size or value            */
#define CPGPU_ERR_CUDA          -2  /* a CUDA runtime call failed                */
#define CPGPU_ERR_CAPACITY      -3  /* a device buffer (pairs, contacts...) overflowed */
#define CPGPU_ERR_NAN           -4  /* a body state became NaN/Inf on the device */
#define CPGPU_ERR_UNSUPPORTED   -5  /* feature outside the implemented path      */
#define CPGPU_ERR_OUT_OF_BUDGET -6  /* serving: request exceeds the HBM budget   */
#define CPGPU_ERR_TIMEOUT       -7  /* a bounded device wait gave up             */
#define CPGPU_ERR_NO_DEVICE     -8  /* no CUDA device / extension not usable     */

/* movement types: RigidBody::MovementType (RigidBody.h:22) */
#define CPGPU_DYNAMIC   0
#define CPGPU_FIXED     1
#define CPGPU_KINEMATIC 2

typedef struct cpgpu_world  cpgpu_world;   /* one PhysicsEngine              */
typedef struct cpgpu_batch  cpgpu_batch;   /* many independent worlds        */
typedef struct cpgpu_server cpgpu_server;  /* continuous-batching rollouts   */

/* Material (ConvexPrimitive.h:17-34).  cfm is always the global one. */
typedef struct cpgpu_material {
    double density;
    double restitution;
    double kinetic_friction;
    double static_friction;
} cpgpu_material;

/* One persistent contact point (PersistentConstraint.h:51-86), as stored in the
 * contact graph after a step.  Used for diagnostics, checkpoints and parity. */
typedef struct cpgpu_contact {
    uint32_t b1, b2;            /* body ids, b1 < b2 (OrderedBodyPair)      */
    uint32_t live;              /* is_live_contact                          */
    int32_t  memory_life;       /* memory_life                              */
    uint64_t magic_c, magic_b;  /* MagicID {cID, bID} (CollisionDetect.h:29) */
    double   p_local_b1[3];     /* contact_pos_local_b1                     */
    double   p_local_b2[3];     /* contact_pos_local_b2                     */
    double   n_local_b1[3];     /* normal_local_b1                          */
    double   pen_depth;
    double   bounce;
    double   friction_coeff;
    double   normal_impulse;    /* contact.impulse                          */
    double   friction_impulse[2];
    double   friction_u[3];     /* friction.u / friction.w of the last row  */
    double   friction_w[3];
    uint32_t static_ready;      /* friction.getStaticReady()                */
    uint32_t pad_;
} cpgpu_contact;

/* ---- world lifetime and parameters ------------------------------------- */
/* PhysicsEngine::PhysicsEngine() with the defaults of PhysicsEngine.h:170-227 */
int cpgpu_world_create(cpgpu_world** out);
/* PhysicsEngine::~PhysicsEngine (PhysicsEngine.cpp:31-37).  A world that a
 * live batch was made from is freed when the last such batch is destroyed
 * (the handle must not be used after this call either way). */
int cpgpu_world_destroy(cpgpu_world* w);
/* PhysicsEngine::setStep_time (PhysicsEngine.cpp:1214-1217) */
int cpgpu_set_step_time(cpgpu_world* w, double dt);
/* PhysicsEngine::setGravity (PhysicsEngine.cpp:1142-1145) */
int cpgpu_set_gravity(cpgpu_world* w, double gx, double gy, double gz);
/* PhysicsEngine::setSubstepCount (PhysicsEngine.h:91) */
int cpgpu_set_substep_count(cpgpu_world* w, int substeps);
/* PhysicsEngine::setPGSIterations (PhysicsEngine.h:90) */
int cpgpu_set_pgs_iterations(cpgpu_world* w, int n_vel, int n_pos, int n_holonomic);
/* PhysicsEngine::setSleepingEnabled (PhysicsEngine.cpp:1138-1140).  Worlds
 * start with sleeping disabled (the reference's default is enabled); bodies
 * already asleep stay asleep until woken when it is disabled again, as in the
 * reference.  Sleeping follows PhysicsEngine.cpp:65-87, 174, 1113-1136,
 * 1221-1290 and 1536-1613; where the reference's outcome depends on an
 * unordered_map's iteration order (a sleeping island that one body wakes
 * while another would have been stopped), a wake takes precedence. */
int cpgpu_set_sleeping_enabled(cpgpu_world* w, int enabled);
/* PhysicsEngine::setWarmStartDisabled (PhysicsEngine.cpp:1182-1184) */
int cpgpu_set_warm_start_disabled(cpgpu_world* w, int disabled);
/* PhysicsEngine::setGlobalConstraintForceMixing (PhysicsEngine.cpp:1193-1195) */
int cpgpu_set_global_cfm(cpgpu_world* w, double cfm);
/* PhysicsEngine::setAngleVelUpdateTickCount (PhysicsEngine.cpp:1173-1176) */
int cpgpu_set_angle_vel_update_tick_count(cpgpu_world* w, int n);
/* PhysicsEngine::setInternalGyroscopicForcesDisabled (PhysicsEngine.cpp:1178-1180) */
int cpgpu_set_internal_gyro_forces_disabled(cpgpu_world* w, int disabled);

/* ---- bodies ------------------------------------------------------------- */
/* createRigidBody(ConvexUnionGeometry(Polyhedron(points, faces), material),
 * movement, position) (PhysicsEngine.cpp:486-496, ConvexPrimitive.h:212).
 * points: n_points xyz; faces: CSR (face_offsets has n_faces+1 entries). */
int cpgpu_body_hull(cpgpu_world* w, const double* points, int n_points,
                    const int* face_offsets, const int* face_indices, int n_faces,
                    const cpgpu_material* mat, int movement, const double pos[3],
                    uint32_t* out_id);
/* createRigidBody(ConvexUnionGeometry::box(corner, dx, dy, dz, material), ...)
 * (Geometry.cpp:14-37) */
int cpgpu_body_box(cpgpu_world* w, const double corner[3], double dx, double dy, double dz,
                   const cpgpu_material* mat, int movement, const double pos[3],
                   uint32_t* out_id);
/* createRigidBody(ConvexUnionGeometry::sphere(center, radius, material), ...)
 * (Geometry.cpp:39-41) */
int cpgpu_body_sphere(cpgpu_world* w, const double center[3], double radius,
                      const cpgpu_material* mat, int movement, const double pos[3],
                      uint32_t* out_id);
/* createRigidBody(ConvexUnionGeometry::cylinder(base, radius, height, material), ...)
 * (Geometry.cpp:47-49) */
int cpgpu_body_cylinder(cpgpu_world* w, const double base[3], double radius, double height,
                        const cpgpu_material* mat, int movement, const double pos[3],
                        uint32_t* out_id);
/* createRigidBody(ConvexUnionGeometry::capsule(bot_sphere_center, radius,
 * drum_height, material), ...) (Geometry.cpp:43-45): `bot` is the centre of
 * the bottom cap sphere, `drum_height` the distance between the two cap-sphere
 * centres, the height axis +y.  Pairs: SAT_PolyCapsule, detectSphereCapsule,
 * detectCapsuleCapsule, detectCapsuleCylinder, SAT_CapsuleTriangle
 * (CollisionDetect.cpp:1413-1561, 868-935, 1139-1334, 1794-2002, 2278-2464). */
int cpgpu_body_capsule(cpgpu_world* w, const double bot[3], double radius, double drum_height,
                       const cpgpu_material* mat, int movement, const double pos[3],
                       uint32_t* out_id);
/* One primitive of a multi-primitive body (ConvexUnionGeometry, Geometry.h:9-47). */
#define CPGPU_PRIM_HULL 0
#define CPGPU_PRIM_BOX 1
#define CPGPU_PRIM_SPHERE 2
#define CPGPU_PRIM_CYLINDER 3
#define CPGPU_PRIM_CAPSULE 4
typedef struct cpgpu_primitive {
    int kind;               /* CPGPU_PRIM_* */
    double p[3];            /* box corner, sphere centre, cylinder base, capsule bottom-sphere centre */
    double a, b, c;         /* box dx dy dz; sphere radius; cylinder radius, height; capsule radius, drum height */
    const double* points;   /* hull: points (xyz) and faces as for cpgpu_body_hull */
    int n_points;
    const int* face_offsets;
    const int* face_indices;
    int n_faces;
    cpgpu_material mat;
} cpgpu_primitive;
/* createRigidBody(ConvexUnionGeometry::merge(...) of the n primitives in
 * order, movement, pos) (Geometry.cpp:540-550, RigidBody.cpp:13-39): mass
 * properties summed over the primitives, each primitive its own AABB and
 * material, pairs of bodies tested primitive pair by primitive pair
 * (PhysicsEngine.cpp:182-219), their manifolds merged and culled per body
 * pair (PhysicsEngine.cpp:257-295).  n = 1 is the same as the
 * single-primitive calls; at most 255 primitives per body. */
int cpgpu_body_union(cpgpu_world* w, const cpgpu_primitive* prims, int n, int movement, const double pos[3],
                     uint32_t* out_id);
/* createRigidBody(StaticMeshGeometry(MeshInput{tris, points}), fixed)
 * (PhysicsEngine.cpp:498-512, Geometry.h:52-55): points (xyz) and triangles
 * (three point indices each) in world coordinates, fewer than 2^24
 * triangles; `fixed` must be nonzero (kinematic meshes:
 * CPGPU_ERR_UNSUPPORTED).  Mesh-mesh pairs never collide. */
int cpgpu_body_mesh(cpgpu_world* w, const double* points, int n_points,
                    const int* tris, int n_tris, const cpgpu_material* mat,
                    int fixed, uint32_t* out_id);

/* RigidBody::setVel / setAngVel / setOrientation / setToPosition / setMass
 * (RigidBody.cpp:69-118) */
int cpgpu_body_set_velocity(cpgpu_world* w, uint32_t id, const double v[3]);
int cpgpu_body_set_ang_velocity(cpgpu_world* w, uint32_t id, const double v[3]);
int cpgpu_body_set_orientation(cpgpu_world* w, uint32_t id, const double q[4]);
int cpgpu_body_set_position(cpgpu_world* w, uint32_t id, const double p[3]);
int cpgpu_body_set_mass(cpgpu_world* w, uint32_t id, double mass);

/* ---- holonomic constraints --------------------------------------------- */
/* PhysicsEngine::addBallSocketConstraint (PhysicsEngine.cpp:664-687) */
int cpgpu_add_ball_socket(cpgpu_world* w, uint32_t b1, uint32_t b2,
                          const double b1_attach_local[3], const double b2_attach_local[3],
                          double pos_correct_strength, uint32_t* out_id);
/* PhysicsEngine::addDistanceConstraint (PhysicsEngine.cpp:623-660): the
 * attachment points stay `target_distance` apart (-1: their distance at
 * creation); DistanceConstraint rows (ConstraintSolver.cpp:348-377). */
int cpgpu_add_distance(cpgpu_world* w, uint32_t b1, uint32_t b2,
                       const double b1_attach_local[3], const double b2_attach_local[3],
                       double target_distance, double pos_correct_strength, uint32_t* out_id);
/* PhysicsEngine::addWeldConstraint (PhysicsEngine.cpp:892-915): the two
 * bodies move as one about the attachment points; WeldConstraint rows
 * (ConstraintSolver.cpp:861-899). */
int cpgpu_add_weld(cpgpu_world* w, uint32_t b1, uint32_t b2,
                   const double b1_attach_local[3], const double b2_attach_local[3],
                   double pos_correct_strength, double rot_correct_strength, uint32_t* out_id);
/* PhysicsEngine::addTwistLimitConstraint (PhysicsEngine.cpp:948-972): the
 * twist of body 2 about the axes stays within [min_angle, max_angle];
 * TwistLimitConstraint row (ConstraintSolver.cpp:439-466). */
int cpgpu_add_twist_limit(cpgpu_world* w, uint32_t b1, uint32_t b2,
                          const double b1_twist_axis_local[3], const double b2_twist_axis_local[3],
                          double min_angle, double max_angle, double rot_correct_strength, uint32_t* out_id);
/* PhysicsEngine::addConeLimitConstraint (PhysicsEngine.cpp:922-946): the
 * angle between the bodies' direction vectors (body space) stays below
 * max_angle (< pi); ConeLimitConstraint row (ConstraintSolver.cpp:410-436). */
int cpgpu_add_cone_limit(cpgpu_world* w, uint32_t b1, uint32_t b2,
                         const double b1_cone_direction_local[3], const double b2_cone_direction_local[3],
                         double max_angle, double rot_correct_strength, uint32_t* out_id);
/* PhysicsEngine::addSpring (PhysicsEngine.cpp:974-998): a damped spring
 * between the attachment points (resting_length < 0: their distance at
 * creation), applied as impulses at the start of every substep
 * (PhysicsEngine.cpp:1313-1356). */
int cpgpu_add_spring(cpgpu_world* w, uint32_t b1, uint32_t b2,
                     const double b1_attach_local[3], const double b2_attach_local[3],
                     double damping, double stiffness, double resting_length, uint32_t* out_id);
/* PhysicsEngine::addSliderConstraint (PhysicsEngine.cpp:769-806): body 2
 * slides along body 1's axis without turning; SliderConstraint rows
 * (ConstraintSolver.cpp:611-696). */
int cpgpu_add_slider(cpgpu_world* w, uint32_t b1, uint32_t b2,
                     const double b1_slider_pos_local[3], const double b2_slider_pos_local[3],
                     const double b1_slider_axis_local[3], const double b2_slider_axis_local[3],
                     double pos_correct_strength, double rot_correct_strength, uint32_t* out_id);
/* PhysicsEngine::addSlidingHingeConstraint (PhysicsEngine.cpp:856-890): body
 * 2 slides along and turns about the shared axis; SlidingHingeConstraint rows
 * (ConstraintSolver.cpp:781-852). */
int cpgpu_add_sliding_hinge(cpgpu_world* w, uint32_t b1, uint32_t b2,
                            const double b1_slider_pos_local[3], const double b2_slider_pos_local[3],
                            const double b1_slider_axis_local[3], const double b2_slider_axis_local[3],
                            double pos_correct_strength, double rot_correct_strength, uint32_t* out_id);
/* PhysicsEngine::addHingeConstraint (PhysicsEngine.cpp:693-723) */
int cpgpu_add_hinge(cpgpu_world* w, uint32_t b1, uint32_t b2,
                    const double b1_attach_local[3], const double b2_attach_local[3],
                    const double b1_axis_local[3], const double b2_axis_local[3],
                    double pos_correct_strength, double rot_correct_strength,
                    uint32_t* out_id);
/* PhysicsEngine::addMotorConstraint (PhysicsEngine.cpp:725-763): a motor on
 * the hinge or sliding hinge `base_id` (its axes and rotation strength), with
 * angle limits (-inf / +inf for none).  Off until set_motor powers it; its
 * row is solved while powered or past a limit. */
int cpgpu_add_motor(cpgpu_world* w, uint32_t base_id, double min_angle, double max_angle, uint32_t* out_id);
/* PhysicsEngine::addPistonConstraint (PhysicsEngine.cpp:808-852): a piston on
 * the slider or sliding hinge `base_id` (its tracked points, body 1 axis and
 * position strength), with slide limits.  It occupies two consecutive slots
 * of the joint state (its slide limit, then its powered row). */
int cpgpu_add_piston(cpgpu_world* w, uint32_t base_id, double min_pos, double max_pos, uint32_t* out_id);
/* PhysicsEngine::setMotorOff / setMotorConstantTorque / setMotorTargetVelocity
 * / setMotorTargetPosition (PhysicsEngine.cpp:1857-1912) as mode 0 / 1 / 2 / 3:
 * mode 1 sets the torque (max_torque), modes 2 and 3 the max torque and the
 * target velocity or angle; mode 0 leaves them.  Both bodies are woken. */
int cpgpu_set_motor(cpgpu_world* w, uint32_t id, int mode, double max_torque, double target);
/* setPistonOff / setPistonConstantForce / setPistonTargetVelocity /
 * setPistonTargetPosition (PhysicsEngine.cpp:1800-1855), the same for force. */
int cpgpu_set_piston(cpgpu_world* w, uint32_t id, int mode, double max_force, double target);
/* getMotorAngularPosition / getPistonPosition (PhysicsEngine.cpp:1914-1930):
 * the angle (unwrapped) or slide position of the last rebuild. */
int cpgpu_get_motor_position(cpgpu_world* w, uint32_t id, double* out);
int cpgpu_get_piston_position(cpgpu_world* w, uint32_t id, double* out);

/* ---- stepping and state ------------------------------------------------- */
/* n_steps x PhysicsEngine::timeStep (PhysicsEngine.cpp:50-471) */
int cpgpu_step(cpgpu_world* w, int n_steps);
/* PhysicsEngine::getNumBodies (PhysicsEngine.h:86) */
int cpgpu_num_bodies(cpgpu_world* w, int* n);
/* RigidBody::getCOM/getOrientation/getVel/getAngVel for every body in id order;
 * any output pointer may be NULL.  com/vel/ang_vel: 3 doubles per body,
 * quat: 4 doubles (r,i,j,k) per body. */
int cpgpu_get_body_state(cpgpu_world* w, double* com, double* quat, double* vel, double* ang_vel);
/* RigidBody::getAsleep (RigidBody.h:35) for every body in id order:
 * flags[i] = 1 for a dynamic body that is asleep, else 0. */
int cpgpu_get_asleep(cpgpu_world* w, int* flags);
/* Overwrite the dynamic state of every body (a checkpoint restore); any input
 * pointer may be NULL.  The world geometry follows the new poses. */
int cpgpu_set_body_state(cpgpu_world* w, const double* com, const double* quat,
                         const double* vel, const double* ang_vel);
/* RigidBody::getAABB for every body, 6 doubles (min xyz, max xyz) per body */
int cpgpu_get_aabbs(cpgpu_world* w, double* aabbs);
/* Candidate pairs of the last broadphase (AABBTree::getAllCollisionCandidates,
 * AABB_Tree.h:153-224) as (lower id, higher id), sorted; *n receives the count,
 * at most cap pairs are written. */
int cpgpu_get_pairs(cpgpu_world* w, uint32_t* pairs, int cap, int* n);
/* Every persistent contact of the contact graph, sorted by (b1, b2) and in the
 * per-edge order of SharedConstraintsEdge::constraints (PhysicsEngine.h:248). */
int cpgpu_get_contacts(cpgpu_world* w, cpgpu_contact* out, int cap, int* n);
/* Replace the whole contact graph (a checkpoint restore).  Same layout and
 * order as cpgpu_get_contacts. */
int cpgpu_set_contacts(cpgpu_world* w, const cpgpu_contact* in, int n);
/* PhysicsEngine::raycastFirstIntersection (PhysicsEngine.cpp:582-609) for
 * n_rays rays at once.  Ray k starts at origins[3k..3k+2] with the unit
 * direction dirs[3k..3k+2]; the bodies whose ids are listed in `ignore`
 * (n_ignore of them) are skipped.  Every body whose current AABB the ray
 * crosses (AABB::rayIntersectsAABB, AABB.h:143-172) is tested with its
 * primitive's ray test (RigidBody::checkRayIntersection, RigidBody.cpp:185-204;
 * ConvexPrimitive.cpp:113-212, 300-318, 403-411, 445-447, 731-758;
 * Geometry.cpp:867-897) and the nearest hit wins.  The reference filters with
 * its broadphase tree, whose leaves hold the AABBs of the start of the last
 * step; this call uses the current ones.  Outputs per ray (any may be NULL):
 * hit_body (0: no hit), hit_pos (3), hit_normal (3), hit_dist (-1: no hit). */
int cpgpu_raycast(cpgpu_world* w, const double* origins, const double* dirs, int n_rays,
                  const uint32_t* ignore, int n_ignore, uint32_t* hit_body,
                  double* hit_pos, double* hit_normal, double* hit_dist);
/* Warm-start state of the joints (not the springs) in creation order: the
 * impulse of each constraint row (PersistentConstraint.h:90-420), 6 doubles
 * per joint (ball-socket 3 used, sliding hinge 4, hinge and slider 5, weld 6,
 * distance, limits, motors and pistons 1); the tangent basis u, w of its last
 * rebuild (hinge, slider, sliding hinge; 3 doubles each); and `aux`, 2
 * doubles per joint: a twist limit's current angle (unwrapped across
 * rebuilds), a motor's angle or a piston's slide position, and then for a
 * cone or twist limit 1 when its last rebuild found the limit reached (the
 * row is then solved in the next step), for a motor the relative angular
 * velocity of its last rebuild, for a piston's two slots 1 when past a slide
 * limit, else 0.  With the body state and the
 * contacts this completes a checkpoint; no counterpart in the reference,
 * which keeps these inside its constraint objects.  Any pointer but `n` may
 * be NULL. */
int cpgpu_get_joint_state(cpgpu_world* w, double* impulse, double* u, double* wv, double* aux, int* n);
int cpgpu_set_joint_state(cpgpu_world* w, const double* impulse, const double* u, const double* wv, const double* aux,
                          int n);

/* ---- batched worlds ----------------------------------------------------- */
/* Pack independent worlds into one device batch (segmented arrays) that one
 * launch sequence per step advances.  The worlds keep their own state; the
 * batch starts from their current state and the substep count must agree.
 * The batch holds on to the worlds (cpgpu_world_destroy frees them only with
 * the batch): the autotuner re-packs the batch from their descriptions. */
int cpgpu_batch_create(cpgpu_world* const* worlds, int n_worlds, cpgpu_batch** out);
/* Autotuner (no counterpart in the reference): re-chooses the batch's
 * schedule by timing from its current state.  Candidate schedules -- one to
 * four parts with several shares of the bodies in the parts of the largest
 * worlds; for each, the later parts' solver-chain workers per SM and the
 * island size from which an island takes the warp-per-island solver -- are
 * built from the current state, timed on `trial_steps` steps run together
 * and as many steps run one at a time (the score is the mean of the two
 * per-step times), the state restored after each trial, and the fastest
 * adopted; the batch continues from exactly the state it had, and the
 * worlds' own state is not touched.  In calls of several steps, each part's
 * pair, narrowphase and island stages follow those of the part before it
 * (the parts of the largest worlds reach their solver chains first) and the
 * rest of the parts' steps run concurrently; a single step runs the parts
 * fully concurrently.  CPGPU_ERR_INVALID_ARG if a world was changed through
 * the API after the batch was made from it.  Tune from a representative
 * state (e.g. after some steps: before bodies touch, a step costs far
 * less).  The choice is cached per world-size histogram (log2 bins of the
 * body counts), for the process and, when the environment variable
 * CPGPU_TUNE_FILE names a file, there; cpgpu_batch_create uses a cached
 * choice for a matching histogram unless CPGPU_BATCH_PARTS,
 * CPGPU_BATCH_FIRST_SHARE, CPGPU_BATCH_SECOND_SHARE, CPGPU_PGS_REST_PER_SM,
 * CPGPU_PGS_MID_PER_SM or CPGPU_PGS_BIG_ROWS is set (CPGPU_BATCH_STAGGER=0
 * runs the parts fully concurrently in calls of several steps too;
 * CPGPU_PGS_DV_CAP caps the island bodies whose solver Δv stays in shared
 * memory, 1536 by default).  Every world steps exactly
 * as it does alone under any schedule. */
int cpgpu_batch_tune(cpgpu_batch* b, int trial_steps);
/* cpgpu_batch_create followed by cpgpu_batch_tune from the worlds' state. */
int cpgpu_batch_create_tuned(cpgpu_world* const* worlds, int n_worlds, int trial_steps, cpgpu_batch** out);
/* The batch's schedule: sched[6] = parts, first-part share of the bodies (%),
 * chain workers per SM of the later parts (0 = as many as fit), big-island row
 * threshold, 1 if chosen by the autotuner, second-part share (%, 0: the
 * parts after the first split the rest evenly); times[2] = the tuned schedule's and
 * the hand-set schedule's scores measured while tuning (device ms per step,
 * the mean of a step inside a run of steps and a step run alone; -1 when not
 * tuned here).  Either pointer may be NULL. */
int cpgpu_batch_schedule(cpgpu_batch* b, int* sched, double* times);
int cpgpu_batch_destroy(cpgpu_batch* b);
int cpgpu_batch_step(cpgpu_batch* b, int n_steps);
/* Body state of world `world_index` of the batch (same layout as above). */
int cpgpu_batch_get_body_state(cpgpu_batch* b, int world_index, double* com, double* quat,
                               double* vel, double* ang_vel);
/* Total bodies, worlds and live contact points of the batch. */
int cpgpu_batch_info(cpgpu_batch* b, int64_t* n_bodies, int64_t* n_worlds, int64_t* n_contacts);

/* Device time of n_steps of the batch (CUDA events on the batch's stream). */
int cpgpu_batch_step_timed(cpgpu_batch* b, int n_steps, double* device_ms);
/* Whole-batch state transfer in the device layout: 16 floats per body
 * (com xyz, inverse mass, quaternion r i j k, velocity xyz + pad, angular
 * velocity xyz + pad), bodies in batch order.  Writing takes the velocities
 * as given; bodies whose pose changed get their world inertia tensors and
 * AABBs recomputed (unchanged bodies keep them exactly, so a read/write round
 * trip does not perturb the simulation); the inverse mass slot is ignored on
 * write and the contact graph is kept. */
int cpgpu_batch_read_state(cpgpu_batch* b, float* out);
int cpgpu_batch_write_state(cpgpu_batch* b, const float* in);
/* Per-stage device time of n_steps run stage by stage (no graph, the parts
 * of the batch concurrent, one step at a time), for the roofline: stage_ms
 * receives CPGPU_N_STAGES totals in the order gravity, pairs, narrowphase,
 * merge, islands, rows, pgs, integrate, geometry, each step's stage time
 * being the time some part of the batch spends in the stage (the union of
 * the parts' intervals in it, so no stage exceeds the step); counts (may be
 * NULL) receives the last step's pairs, contacts and islands summed over the
 * parts. */
#define CPGPU_N_STAGES 9
int cpgpu_batch_profile(cpgpu_batch* b, int n_steps, double* stage_ms, int64_t* counts);
/* The same stage-by-stage steps (one at a time, the parts concurrent),
 * reported per batch part: out[p * n_marks + m] receives the mean ms from
 * the step's start to mark m of part p: mark 0 the part's start, marks 1-5
 * the ends of gravity, pairs, narrowphase, merge and islands with the PGS
 * schedule, then per substep the ends of rows, PGS and integration, and last
 * the end of geometry (n_marks = 7 + 3 * substeps).  With out == NULL only
 * n_parts and n_marks are written; cap is out's length in doubles. */
int cpgpu_batch_timeline(cpgpu_batch* b, int n_steps, double* out, int cap, int* n_parts, int* n_marks);
/* Number of kernel launches one step of the batch issues. */
int cpgpu_batch_launches_per_step(cpgpu_batch* b, int* n);

/* ---- FP64 momentum / energy audit --------------------------------------- */
/* No counterpart in the reference (which computes in FP64 throughout).  When
 * enabled, every step ends with a device pass that sums, per world and in
 * FP64 over the FP32 state, CPGPU_AUDIT_VALUES values:
 *   [0..2] linear momentum sum(m v)
 *   [3..5] angular momentum about the origin sum(x × m v + I_world ω)
 *   [6]    kinetic energy sum(m |v|^2 / 2 + ω·I_world ω / 2)
 *   [7]    gravitational potential energy -sum(m g·x)
 *   [8]    largest increase of [6] + [7] over one step since enabled
 *   [9]    steps audited since enabled
 * over the dynamic bodies (fixed and kinematic ones are left out).  Enabling
 * resets the values; the read returns those of the last step. */
#define CPGPU_AUDIT_VALUES 10
int cpgpu_world_set_audit(cpgpu_world* w, int enabled);
int cpgpu_world_read_audit(cpgpu_world* w, double* out);               /* 10 doubles */
int cpgpu_batch_set_audit(cpgpu_batch* b, int enabled);
int cpgpu_batch_read_audit(cpgpu_batch* b, double* out);               /* 10 per world, batch order */

/* ---- allocation-free pair generation ------------------------------------ */
/* No counterpart in the reference (its broadphase is the AABB tree inside
 * PhysicsEngine::timeStep).  For callers that cannot allocate device memory
 * when they need the broadphase -- code living inside another framework's
 * memory pool, real-time loops that must not enter the driver's allocator,
 * plugins handed only pre-allocated buffers -- this computes the same
 * candidate pairs as the device path's pair generation for one set of AABBs
 * and allocates nothing: every buffer is the caller's device memory, and the
 * only scratch is a fixed file-scope device array (about 260 KB, held by
 * every GPU that loads the library until the process exits).
 *   aabbs   device, n_bodies x 6 floats (min xyz, max xyz)
 *   pairs   device, cap x 2 uint32: (i, j) with 1-based ids, i < j, sorted
 *   count   device int: number of overlapping pairs (may exceed cap; only
 *           the first cap are written)
 *   stream  cudaStream_t (NULL: the default stream)
 * n_bodies may be at most 65536; larger sizes return CPGPU_ERR_INVALID_ARG
 * with a message.  The first call on a device looks up the scratch array's
 * device address (with that device current), so make that first call before
 * any stream capture.  Every call on a device shares the scratch array, so
 * calls whose executions overlap on the GPU (different streams without
 * ordering) race; calls ordered on one stream are safe.  Each call rewrites
 * all the scratch it reads.  The scratch address is cached per CUDA context,
 * so a device reset by the caller is followed by a fresh lookup.  Errors:
 * CPGPU_ERR_INVALID_ARG (sizes, NULL buffers), CPGPU_ERR_NO_DEVICE,
 * CPGPU_ERR_CUDA when a CUDA error from earlier work is already pending on
 * the thread (left pending, nothing launched) or when one of this call's
 * launches fails; kernel faults surface at the caller's next synchronisation. */
int cpgpu_pairs_noalloc(const float* aabbs, int n_bodies, uint32_t* pairs, int cap, int* count, void* stream);

/* ---- serving ------------------------------------------------------------- */
/* A copy of a world (bodies, shapes, joints, parameters, contact graph, the
 * same node-map order); the copy steps exactly as the original would.  For
 * rollout services that instantiate many requests from a few templates.  No
 * counterpart in the reference. */
int cpgpu_world_clone(cpgpu_world* src, cpgpu_world** out);

/* Continuous-batching rollout server (no counterpart in the reference).  A
 * request is a world plus a number of steps.  Requests are sorted by size
 * into lanes (fewer than 128 dynamic bodies, fewer than 512, the rest); in
 * each lane they wait in arrival order until their estimated device memory
 * fits the one budget next to all running requests, and a lane's running
 * requests are stepped together as one batch on the lane's own stream, their
 * state resident on the device between admission points.  A lane's batch is
 * re-formed when its finished requests hold a quarter of its bodies, or when
 * requests wait and `epoch_steps` steps have passed since its last re-form; a
 * completed request's final state is written back into its world, which the
 * caller then reads as usual.  Each request's result equals stepping its
 * world alone.  The caller must not touch a submitted world until its token
 * is returned by cpgpu_server_poll. */
int cpgpu_server_create(int64_t hbm_budget_bytes, int epoch_steps, cpgpu_server** out);
int cpgpu_server_destroy(cpgpu_server* s);
int cpgpu_server_submit(cpgpu_server* s, cpgpu_world* w, int steps, uint64_t* token);
/* Launch up to max_steps steps on every idle lane (never past a running
 * request's remaining count) and return once one lane's launched steps have
 * completed, or at once when nothing runs; lanes progress at their own pace. */
int cpgpu_server_advance(cpgpu_server* s, int max_steps, int* n_running, int* n_waiting);
/* Tokens of requests completed since the last poll. */
int cpgpu_server_poll(cpgpu_server* s, uint64_t* tokens, int cap, int* n);
/* Totals: body-steps advanced, batch re-forms and their host time (ms),
 * device bytes of the lanes' current batches, bodies running. */
int cpgpu_server_stats(cpgpu_server* s, int64_t* body_steps, int64_t* reforms, double* reform_ms,
                       int64_t* device_bytes, int64_t* running_bodies);

/* ---- diagnostics -------------------------------------------------------- */
/* Last error message of this thread (static storage, never NULL). */
const char* cpgpu_last_error(void);

#ifdef __cplusplus
}
#endif

#endif /* CPGPU_H */
