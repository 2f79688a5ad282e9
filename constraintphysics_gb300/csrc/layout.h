// layout.h — device data layout of the GB300 contact path (shared by the host
// engine and the kernels).
//
// One "batch" holds any number of independent worlds in segmented
// structure-of-arrays buffers: bodies of world w occupy the contiguous global
// index range [world_body_start[w], world_body_start[w+1]); a single world is a
// batch of one.  Everything a step touches lives in HBM; per-step sizes (pairs,
// edges, contacts, islands) are device-side counters so the whole step can be
// captured once in a CUDA graph and replayed.
#pragma once
#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

namespace cpgpu {

// ---- packed convex-hull blob -------------------------------------------------
// 16-byte aligned, size a multiple of 16 B, copied into shared memory with one
// bulk copy.  All geometry is in the body's reference frame (centred on the
// centre of mass), FP32.  Section offsets are in bytes from the blob start.
struct alignas(16) HullHeader {
    uint16_t nv, nf, ne, na;       // vertices, faces, edges, Gauss arcs
    uint16_t nfi, size16;          // face-index count, blob size in 16 B units
    uint16_t off_norm, off_cache;  // float4 sections
    uint16_t off_fofs, off_fidx;   // face CSR (uint16 offsets, uint8 vertex ids)
    uint16_t off_edge, off_arc;    // uint8 pairs
    uint16_t off_vfofs, off_vfidx; // vertex -> adjacent faces CSR
    uint16_t off_veofs, off_veidx; // vertex -> adjacent edges CSR
    uint32_t kind;                 // ShapeKind
    float radius;                  // bound on |vertex| (reference frame)
    uint32_t pad[2];
};
static_assert(sizeof(HullHeader) == 48, "hull header size");
// verts follow the header: float4 {x, y, z, 0} x nv
// norm:  float4 {nx, ny, nz, redundant ? 1 : 0} x nf  (Gauss-map vertices)
// cache: float4 {max, min, bits(max_id), bits(min_id)} x nf: extrema of the hull
//        along its own face normal, in the reference frame; the world value adds
//        dot(R n, com) (the recentring of CollisionDetect.cpp:622-625)
// ---- sphere and cylinder blobs ------------------------------------------------
// Same header (kind 1 = sphere, 2 = cylinder, 4 = capsule; nv = nf = ne = na = 0; the whole
// blob is the hot part, off_fofs = its size), then, in the reference frame:
//   float4 c      {centre xyz, radius}
// cylinders only (Cylinder, ConvexPrimitive.h:160-210; 12 Gauss ring vertices,
// 8-gon cap approximations):
//   float4 axis   {height axis xyz, height}
//   float4 gv[14] Gauss vertices: caps (+axis, -axis), then the ring
//   float4 top[8] top-cap 8-gon
//   float4 bot[8] bottom-cap 8-gon
// capsules only (Capsule, ConvexPrimitive.h:107-141; kind 4):
//   float4 c      {centre xyz, radius}
//   float4 axis   {height axis xyz, drum height (distance of the cap-sphere centres)}
enum ShapeKind : uint32_t { SHAPE_HULL = 0, SHAPE_SPHERE = 1, SHAPE_CYLINDER = 2, SHAPE_MESH = 3, SHAPE_CAPSULE = 4 };
constexpr int kCylRing = 12, kCylCap = 8;
constexpr int kCylOffAxis = 64, kCylOffGv = 80, kCylOffTop = 80 + 16 * 14, kCylOffBot = 80 + 16 * 22;
constexpr int kSphereBlob = 64, kCylBlob = 80 + 16 * 30, kCapBlob = 80;

// ---- static triangle mesh blob (kind 3; world coordinates; read from global,
// never staged).  Header pad[0] = triangles, pad[1] = tree nodes (root first):
//   float4 lo, hi                  mesh AABB
//   nodes: float4 lo (w: left child, bits; -1 = leaf), float4 hi (w: right
//          child or, for a leaf, the triangle index, bits)
//   triangles, kMeshTriF4 float4 each: normal (w: concave-neighbour count,
//          bits), v0, v1, v2 (w: unused), out0..2 (outward edge directions),
//          g0..2 (Gauss region; g0.w: its size, bits), ids (edge ids 0..2,
//          triangle id, bits), aabb lo, hi
constexpr int kMeshTriF4 = 13;
constexpr int kMeshOffNodes = 80;
// per-pair limits of the mesh narrowphase (exceeding one sets ST_MESH_OVERFLOW)
constexpr int kMeshCand = 128;   // candidate triangles
constexpr int kMeshMans = 64;    // triangle manifolds
constexpr int kMeshRaw = 256;    // their points before the merge and cull
constexpr int kMeshOut = 64;     // contact points after it
constexpr int kMeshStack = 64;   // tree traversal depth

// per-warp scratch of the mesh narrowphase (global memory, one per resident warp)
struct alignas(16) MeshScratch {
    float4 pt[kMeshRaw];               // raw points: xyz, w pen
    float4 man_n[kMeshMans];           // triangle manifold normal, w its pen
    float4 out_n[kMeshOut];            // normal of each kept point's merged manifold
    unsigned long long magic[kMeshRaw];
    int tri[kMeshRaw];                 // triangle id of each raw point
    int man_first[kMeshMans], man_cnt[kMeshMans];
    int cand[kMeshCand];
    int out[kMeshOut];                 // kept raw points
};

constexpr int kMaxHullVerts = 255;   // uint8 vertex ids
constexpr int kMaxHullFaces = 255;
constexpr int kMaxHullEdges = 255;
constexpr int kMaxHullBlob = 16384; // bytes; bigger hulls are rejected

// ---- per-world parameters (PhysicsEngine.h:170-227) ---------------------------
struct WorldParams {
    float dt, dt_sub;
    float gx, gy, gz;
    float cfm;
    float cutoff_vel;            // 2 |g| dt (PhysicsEngine.h:203)
    float hardness;              // contact_pos_correct_hardness
    int contact_life;
    int angle_ticks;
    int gyro_disabled;
    int warm_disabled;
    int pgs_vel, pgs_pos;
    int pgs_holo;                // holonomic block-solve iterations (first substep)
    // sleeping (PhysicsEngine.h:219-224, PhysicsEngine.cpp:1221-1290): the
    // thresholds as the reference forms them from its coefficients and |g|,
    // and the step counts the host derives from its FP64 time arithmetic
    int sleeping;                // 1: enabled
    int hist_len;                // velocity history kept: (int)(sleep_delay / dt) steps
    int hist_min;                // fewest recorded steps for bodySleepy: !(2 n < sleep_delay / dt)
    int ready_steps;             // sleepy steps for readyToSleep: sleep_delay reached summing dt in FP64
    int non_sleepy_threshold;
    float vel_eps, ang_vel_eps, accel_eps, ang_accel_eps;
    float wake_vel;              // a sleeping body faster than this after a solve wakes its island
};

// ---- status word bits ----------------------------------------------------------
enum StatusBits : int {
    ST_PAIR_OVERFLOW = 1, ST_EDGE_OVERFLOW = 2, ST_CONTACT_OVERFLOW = 4,
    ST_NAN = 8, ST_TIMEOUT = 16, ST_CLIP_OVERFLOW = 32, ST_STACK_OVERFLOW = 64, ST_MESH_OVERFLOW = 128,
};

// contact state word: bits 0-7 life (int8), bit 8 live, bit 9 static_ready, bit 10 dead
__host__ __device__ inline int cs_life(int s) { return (int)(int8_t)(s & 0xff); }
__host__ __device__ inline bool cs_live(int s) { return (s >> 8) & 1; }
__host__ __device__ inline bool cs_static(int s) { return (s >> 9) & 1; }
__host__ __device__ inline bool cs_dead(int s) { return (s >> 10) & 1; }
__host__ __device__ inline int cs_make(int life, bool live, bool st, bool dead) {
    return (life & 0xff) | ((int)live << 8) | ((int)st << 9) | ((int)dead << 10);
}

// One persistent contact point (PersistentConstraint.h:51-86), SoA over the
// contact store.  p1/p2/n are local to body 1 / body 2 / body 1.
struct ContactStore {
    uint64_t* magic;     // bID of the MagicID (cID is implied by the edge)
    float4* p1;          // xyz p1_local, w pen_depth
    float4* p2;          // xyz p2_local, w bounce
    float4* n;           // xyz n_local_b1, w friction_coeff
    float4* imp;         // normal impulse, friction impulse u, w, unused
    float4* fu;          // friction basis u of the last rebuild
    float4* fw;          // friction basis w
    int* state;          // cs_* bits
    int* edge;           // owning edge (index in the edge list)
    int* tri;            // mesh triangle id of the cID (0 for convex pairs)
};

struct EdgeStore {
    uint64_t* key;       // (global body a) << 32 | global body b, a < b
    int* cstart;         // first contact
    int* ccount;         // contacts of the edge
};

// Solver row block of one contact (normal row + 2-dof friction row), built each
// substep in island order (ConstraintSolver.cpp:240-343).  384 bytes, 16-byte
// aligned.  After a 96-byte header come twelve 6-vectors (linear xyz, angular
// xyz), 24 bytes apart from byte 96, so that every (x, y), (z, ax), (ay, az)
// component pair sits in one half of a 16-byte word: the solver loads the
// row with 16-byte loads and computes on the pairs with packed FP32
// instructions (fma.rn.f32x2).
struct alignas(16) RowBlock {
    float4 imp;          // accumulated impulses: normal, pseudo normal, friction u, w
    int sa, sb;          // island body slots (-1 = body with infinite mass)
    int contact;         // contact index
    int stat;            // friction static_ready of the last projection
    int ga, gb;          // global body indices
    float bounce, cutoff;
    float tgt_n, tgt_f0, tgt_f1;   // velocity targets (findTargetConstraintValue)
    float fcoeff;
    float nminv, nptarget;
    float kd0, kd1;      // friction impulse change per unit normal impulse: Fm^-1 (J_f M^-1 J_n^T)
    float fmc[4];        // the friction rows' 2x2 effective-mass inverse Fm^-1 by columns: (m00, m10), (m01, m11)
    float nja[6], njb[6], nita[6], nitb[6];          // normal row J and M^-1 J^T (bodies a, b)
    float fja0[6], fjb0[6], fja1[6], fjb1[6];        // friction rows (u, w)
    float fita0[6], fitb0[6], fita1[6], fitb1[6];    // friction M^-1 J^T columns (u, w)
};
static_assert(sizeof(RowBlock) == 384, "row block size");
static_assert(offsetof(RowBlock, nja) == 96, "row vectors start at byte 96");

// Velocity deltas of an island body (the solver's accumulator): 12 floats in
// kDvF4 float4s, v xyz, w xyz, pv xyz, pw xyz (pseudo velocities for the
// position passes); the (v, w) and (pv, pw) 6-vectors split into the same
// component pairs as the rows' vectors
constexpr int kDvF4 = 3;

// One joint row per substep: DegreedConstraint<n> (ConstraintSolver.h:60-144)
// of a DistanceConstraint (n = 1), BallSocketConstraint (3),
// SlidingHingeConstraint (4), HingeConstraint or SliderConstraint (5),
// WeldConstraint (6), ConeLimitConstraint, TwistLimitConstraint or
// SlideLimitConstraint (1, with a one-sided projection), MotorConstraint or
// PistonConstraint (1, bounded by the max torque or force, with a velocity
// target); row-major, sized for n = 6.
constexpr int kJMax = 6;
struct alignas(16) JointRow {
    float ja[kJMax * 6], jb[kJMax * 6];     // [n][6]
    float ita[6 * kJMax], itb[6 * kJMax];   // [6][n]
    float itv[kJMax * kJMax], minv[kJMax * kJMax];
    float target[kJMax], ptarget[kJMax];
    float impulse[kJMax], pimpulse[kJMax], holo[kJMax];
    int n, sa, sb;                          // island body slots (-1: infinite mass)
    int proj;                               // 0 none, 1 impulse >= 0, 2 impulse <= 0 (limits),
                                            // 3 x > 0 ? min(x, lim) : max(x, -lim) (motor, piston)
    float lim;                              // proj 3 bound
    float vt;                               // motor / piston: target = vt - value
    int has_vt;
    int pos;                                // needsPosCorrect: solved in the position passes
};

// Joint kinds (PersistentConstraint.h:90-420).  The limits are inequality
// rows outside the holonomic systems, listed in an island only while active.
enum JointKind : int {
    JK_BALL = 0, JK_HINGE = 1, JK_DISTANCE = 2, JK_WELD = 3, JK_SLIDER = 4, JK_SLIDING_HINGE = 5,
    JK_CONE = 6, JK_TWIST = 7,
    // Motor (PersistentConstraint.h:253-275) on a hinge's or sliding hinge's
    // axis; Piston (:217-251) on a slider's or sliding hinge's axis, held as two
    // joints: its slide limit, then its powered row
    JK_MOTOR = 8, JK_SLIDE_LIMIT = 9, JK_PISTON = 10,
};
__host__ __device__ inline bool jk_limit(int k) { return k == JK_CONE || k == JK_TWIST; }
__host__ __device__ inline bool jk_powered(int k) { return k == JK_MOTOR || k == JK_SLIDE_LIMIT || k == JK_PISTON; }
// rows listed in an island only while their `active` flag is set, outside the
// holonomic systems
__host__ __device__ inline bool jk_conditional(int k) { return jk_limit(k) || jk_powered(k); }

// Static joint description (PhysicsEngine::add*Constraint): anchors are the
// tracked points relative to each body's centre of mass in its body frame;
// axes in body space.
struct JointStore {
    const int* b1;          // global body indices
    const int* b2;
    const int* n;           // dofs of the row
    const int* kind;        // JointKind
    const float4* p1;       // xyz anchor on body 1
    const float4* p2;
    const float4* ax1;      // hinge / slider axis, cone direction, twist axis (body 1 space)
    const float4* ax2;
    const float2* hard;     // pos / rot correction strength
    const float4* par;      // x: distance target or limit max angle / max slide, y: twist / motor min angle, min slide
    const float4* ul;       // twist, motor: body 1's u axis (body space)
    const float4* wl;       //        and w axis
    const float4* power;    // motor / piston: mode (0 off, 1 constant, 2 target velocity, 3 target
                            // position), max torque / force, target velocity, target position
    float* impulse;         // [kJMax] per joint: persistent warm-start impulse
    float4* u;              // hinge / slider / sliding-hinge basis of the last rebuild
    float4* w;
    float* angle;           // twist: current angle, unwrapped across rebuilds; motor: angular position;
                            // slide limit / piston: slide position
    int* active;            // limits: reached at the last rebuild; motor, piston: listed in the next island
    float* aux;             // motor: relative angular velocity of the last rebuild; slide limit /
                            // piston: 1 when past a slide limit at the last rebuild
    JointRow* rows;
};

// Springs (PhysicsEngine::addSpring, PhysicsEngine.cpp:974-998): impulse
// pairs at the start of every substep, per world in the reference's order
// (node-map order, each edge once, the edge's springs in creation order).
struct SpringStore {
    int n;
    const int* b1;          // global body indices
    const int* b2;
    const float4* p1;       // tracked points (body frame, relative to the centre of mass)
    const float4* p2;
    const float4* par;      // damping, stiffness, resting length
    const int* world_start; // [n_worlds + 1] ranges in that order
};

// Joint edges (SharedConstraintsEdge with joints) sorted by key, per world;
// their joints in insertion order; the holonomic system of the edge (or -1).
struct JointEdgeStore {
    const uint64_t* key;    // (global a) << 32 | global b, a < b
    const int* jstart;      // the edge's joints: jlist[jstart .. jstart + jcount)
    const int* jcount;      // 0 for an edge that holds only springs
    const int* jlist;       // joint indices, each edge's in creation order
    const int* sys;
    const int* world_start; // [n_worlds + 1] joint-edge ranges
    const int* world_jstart;// [n_worlds + 1] joint ranges (row-slot offsets)
};

// Holonomic systems (HolonomicSystem, HolonomicBlockSolver.cpp): constraint
// order, block table and vector offsets built on the host; factor storage in
// FP64 when the system's link-mass ratio exceeds 100, FP32 otherwise.
struct HoloStore {
    int n;                  // systems
    const int* cstart;      // [n + 1] into cons / vpos
    const int* cons;        // joint indices in elimination order
    const int* vpos;        // vector offset of each constraint
    const int* degree;
    const int* tstart;      // [n + 1] into table
    const int* table;       // block_location_table (-1 empty)
    const int* lbase;       // per system: first entry in lstart (n + 1 entries each)
    const int* lstart;      // per column: its nonzero blocks below the diagonal in lrow / lloc
    const int* lrow;        //   their rows (ascending)
    const int* lloc;        //   their block offsets
    const int* bstart;      // offset into the FP32 or FP64 pool
    const int* cap;         // block storage (the diagonal scratch follows)
    const int* fp64;
    const int* wstart;      // offset into the solve workspace (degree doubles)
    float* pool32;
    double* pool64;
    double* work;
    int* isl;               // island of the system in this step (-1 none)
};

constexpr int kSchedInts = 1024;
constexpr int kTile = 128;         // bodies per tile of the large-world pair pass
constexpr int kTileWorld = 2048;   // worlds above this many bodies take the tiled pair pass and component-parallel islands
constexpr int kCompArrays = 12;

struct Batch;  // host object, engine.cu

// All device pointers of a batch, passed by value to kernels.
struct Dev {
    int n_worlds, n_bodies;
    int cap_pairs, cap_edges, cap_contacts;
    const WorldParams* wparams;
    const int* world_start;        // [n_worlds + 1]
    const int* map_order;          // bodies of each world in node-map iteration order
    // bodies
    float4 *pos, *rot, *vel, *angv, *pvel, *pangv;   // pos.w = inverse mass
    float *iinv, *iw;              // world inverse inertia / inertia, 9 floats each
    const float *iref, *iinv_ref;  // reference-frame tensors, 9 floats each
    const int* shape;              // byte offset of the body's hull blob
    const int* world;              // world index of the body
    const uint8_t* movement;
    const float4* material;        // restitution, kinetic, static, unused
    float4 *aabb_lo, *aabb_hi;
    int* moved;
    const uint8_t* shapes;         // hull blob pool
    // broadphase
    int* pair_count;               // per body, then exclusive scan
    int* pair_a; int* pair_b;
    int* n_pairs;
    // worlds of more than kTileWorld bodies: their pairs come from tasks over
    // kTile x kTile blocks of the world's (i, j > i) pairs
    int n_tile_tasks;
    const int4* tile_task;         // x world, y i tile, z j tile (>= y), w the world's tile count
    const int* tile_base;          // per world: offset of its (body, j tile) cells in tile_cnt, -1 small world
    int* tile_cnt;                 // per big-world body and j tile: its pairs there, then their prefix
    // islands of worlds above kTileWorld bodies: one DFS per connected
    // component, the components in parallel (kCompArrays ints per body)
    int* comp;
    int* sys_mark;                 // per holonomic system: the component that counted it
    // narrowphase output per pair
    float4* mf_n;                  // normal xyz, w max_pen (<= 0: no manifold)
    int* mf_cnt;
    float4* mf_pt;                 // [4] per pair: pos xyz, w pen
    uint64_t* mf_magic;            // [4] per pair
    int2* mf_feat;                 // hull pairs: features of the minimum axis (vertex of A, of B) for k_clip
    // static meshes (has_mesh == 0: none in the batch).  A mesh pair's points
    // are in the mesh store at mf_ofs[p] (-1: not a mesh pair), mf_cnt[p] of
    // them, each with its merged manifold's normal; mf_n[p].w is their max pen
    int has_mesh, cap_mesh_pts, mesh_warps;
    int* mf_ofs;
    float4 *mm_pt, *mm_n;
    uint64_t* mm_magic;
    int* mm_tri;
    int* mm_count;
    MeshScratch* msc;
    // bodies of several primitives (has_union == 0: none in the batch); their
    // pairs go through the mesh store like mesh pairs, each point's triangle
    // field holding (primitive of the pair's first body << 8 | of its second)
    // (with a mesh: the triangle id | the convex body's primitive << 24)
    int has_union;
    const int* prim_start;         // per body: its first primitive, -1 for a body of one
    const int* prim_count;
    const int* prim_shape;         // per primitive: blob offset in the pool
    const float4* prim_mat;        // per primitive: restitution, kinetic, static friction
    float4 *prim_lo, *prim_hi;     // per primitive: AABB
    // persistent graph (double-buffered by the host)
    EdgeStore e_old, e_new;
    ContactStore c_old, c_new;
    int *n_edges_old, *n_edges_new, *n_contacts_old, *n_contacts_new;
    // merge scratch
    int *surv, *surv_scan, *unm, *unm_scan, *pair_edge, *edge_src, *edge_pair, *edge_cnt;
    int *edge_live, *edge_row;     // islands: live contacts per edge, first row of an emitted edge
    int *scan_tmp;
    // islands
    int* adj_ofs;                  // per body CSR offsets (scratch)
    int* adj_list;                 // other endpoint | edge index (scratch, 2 ints per entry)
    int* adj_cursor;
    int* visited;                  // per body: island-local slot (-1 = not visited)
    int* stack;                    // per world DFS stack (scratch)
    int* isl_count_w;              // islands per world
    int* isl_row_start; int* isl_row_count; int* isl_body_start; int* isl_body_count; int* isl_world;
    int* isl_scan;
    int* g_isl_row_start; int* g_isl_row_count; int* g_isl_body_start; int* g_isl_body_count; int* g_isl_world;
    int* n_islands;
    int* isl_bodies;               // island body lists (global body index), per-world region
    int* row_contact;              // row slot -> contact
    int* row_of_contact;           // contact -> row slot
    RowBlock* rows;
    float4* dv;                    // 4 float4 per island body slot: dv lin, dv ang, dpv lin, dpv ang
    float4* stage;                 // 4 float4 per body: staging of external state writes
    int* big_list; int* small_list;  // island indices split by row count (PGS scheduling)
    int* sched;                    // schedule counters and tables (kSchedInts ints, layout in solver.cu)
    int* cnt;                      // small device counters (merge totals)
    int* status;
    // joints and holonomic systems (n_joints == 0: none in the batch)
    int n_joints, n_joint_edges;
    JointStore jt;
    JointEdgeStore je;
    HoloStore hs;
    int* isl_flags;                // per world-region island: 1 = has joint rows
    int* g_isl_flags;
    int* isl_sys_start; int* isl_sys_count;        // per world-region island
    int* g_isl_sys_start; int* g_isl_sys_count;
    int* isl_sys;                  // system ids in discovery order (per-world region)
    int* joint_list;               // joint islands (PGS scheduling), count in sched[3]
    const int* hs_world_start;     // [n_worlds + 1] holonomic system ranges (island lists)
    float lin_err_threshold;       // excessive_linear_error_torque_threshold
    float4* dv_err;                // 4 float4 per island body: linearisation-error probe
    SpringStore sp;                // springs (sp.n == 0: none in the batch)
    // polls of a bounded mbarrier wait before a kernel gives up and reports
    // ST_TIMEOUT (kDefaultWaitLimit; CPGPU_WAIT_LIMIT lowers it so that a test
    // can make the waits run out without a fault).  The drain of a giving-up
    // warp's own copies always uses kDefaultWaitLimit.
    long long wait_limit;
    // FP64 audit (audit.cu), null when disabled: kAuditValues doubles per world
    double* audit;
    // islands with at least this many rows take the warp-per-island solver,
    // the others the thread-per-island one (a schedule choice: same results)
    int big_rows;
    // sleeping (has_sleep == 0: no world of the batch has it enabled).  Per
    // body: asleep, waking (an API action or a spring impulse since the last
    // step), sleepy-step count, non-sleepy count, and the last hist_cap
    // (velocity, angular velocity) records as a ring (6 floats each)
    int has_sleep, hist_cap;
    int* asleep;
    int* waking;
    int* ready_cnt;
    int* non_sleepy;
    int* hist_n;
    int* hist_head;
    float* hist;
};

// per world: linear momentum xyz, angular momentum about the origin xyz,
// kinetic energy, potential energy, largest one-step increase of their sum
// since the audit was enabled, steps audited
constexpr int kAuditValues = 10;

constexpr long long kDefaultWaitLimit = 1LL << 24;

}  // namespace cpgpu
