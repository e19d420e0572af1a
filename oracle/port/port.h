// Internal types of the CPU restatement of Box2D v3.1.1's world step.
// TEST INFRASTRUCTURE (oracle): the parity reference for the CUDA path and the
// CPU baseline on machines without the reference checkout. Each function in
// the .c files cites the reference file:line it restates
// (packages/forge2d/third_party/box2d/src/...).
#pragma once

#include "f2d_defs.h"
#include "pmath.h"
#include "ptree.h"

#include <pthread.h>

enum
{
	SHAPE_CIRCLE = 0,
	SHAPE_CAPSULE = 1,
	SHAPE_SEGMENT = 2,
	SHAPE_POLYGON = 3,
	SHAPE_CHAIN_SEGMENT = 4,
};

enum
{
	BODY_STATIC = 0,
	BODY_KINEMATIC = 1,
	BODY_DYNAMIC = 2,
};

typedef struct Polygon
{
	v2 vertices[P_MAX_POLY];
	v2 normals[P_MAX_POLY];
	v2 centroid;
	float radius;
	int count;
} Polygon;

typedef struct Geometry
{
	int type;
	// circle: c1 = center; capsule: c1, c2, radius; segment: c1, c2; chain
	// segment: c1, c2 and the ghost vertices g1 (before c1), g2 (after c2)
	v2 c1, c2;
	float radius;
	Polygon poly;
	v2 g1, g2;
	int chainId;
} Geometry;

// distance.h b2SimplexCache: GJK warm start kept per contact
typedef struct SimplexCache
{
	int count;
	uint8_t indexA[3];
	uint8_t indexB[3];
} SimplexCache;

typedef struct MassData
{
	float mass;
	v2 center;
	float rotationalInertia;
} MassData;

typedef struct ManifoldPoint
{
	v2 point;
	v2 anchorA, anchorB;
	float separation;
	float normalImpulse;
	float tangentImpulse;
	float totalNormalImpulse;
	float normalVelocity;
	uint16_t id;
	bool persisted;
} ManifoldPoint;

typedef struct Manifold
{
	v2 normal;
	float rollingImpulse;
	ManifoldPoint points[2];
	int pointCount;
} Manifold;

typedef struct Body
{
	int used;
	int generation;
	int type;
	int enabled;
	// sim (body.h:120-159)
	xform xf;
	v2 center;
	rot rotation0;
	v2 center0;
	v2 localCenter;
	v2 force;
	float torque;
	float invMass, invInertia;
	float minExtent, maxExtent;
	float linearDamping, angularDamping, gravityScale;
	v2 gravity; // gravity of the body's sub-world (the world's when none)
	int sub;	// sub-world index
	float mass, inertia;
	int isBullet, isSpeedCapped, allowFastRotation, isFast, enlargeAABB, fixedRotation;
	// state (body.h:101-113)
	v2 v;
	float w;
	v2 dp;
	rot dq;
	// topology
	int headShape;
	int shapeCount;
	int headChain; // chains on the body, newest first (body.h headChainId)
	int headJoint; // joint key list: (jointId << 1) | edge
	int jointCount;
	float sleepThreshold, sleepTime;
	int enableSleep;
	// constraint-graph membership: bit c set when the body holds a
	// constraint in colour c < P_OVERFLOW (constraint_graph.c bodySet bitsets)
	uint16_t colorMask;
	int moveEventIndex; // this step's move event slot (finalize)
	// solver set and island (body.h:17-90)
	int setIndex, localIndex;
	int islandId, islandPrev, islandNext;
	int headContactKey; // contact edge list: (contactId << 1) | edge
	int contactCount;
	int isMarked;
} Body;

typedef struct Shape
{
	int used;
	int generation;
	int bodyId;
	Geometry g;
	float density, friction, restitution, rollingResistance, tangentSpeed;
	int userMaterialId;
	uint64_t categoryBits, maskBits;
	int groupIndex;
	int isSensor, enableContactEvents, enableHitEvents, enableSensorEvents, enablePreSolveEvents;
	box2 aabb, fatAABB;
	int sub; // sub-world of the owning body
	int enlarged;
	int moved; // in the move buffer (broad_phase.h:74-82)
	int proxyKey;
	v2 localCentroid;
	int nextShape, prevShape;
	int sensorIndex; // P_NULL unless a sensor
} Shape;

enum
{
	SIM_TOUCHING = 0x00010000,
	SIM_DISJOINT = 0x00020000,
	SIM_STARTED = 0x00040000,
	SIM_STOPPED = 0x00080000,
	SIM_HIT_EVENT = 0x00100000,
	SIM_PRESOLVE = 0x00200000,
};

typedef struct Contact
{
	int used;
	int shapeA, shapeB;
	int bodyA, bodyB;
	int touchingFlag;	  // b2_contactTouchingFlag on b2Contact
	int enableContactEvents; // b2_contactEnableContactEvents
	uint32_t simFlags;
	int color;		   // -1 when not touching
	int overflowIndex; // position in the overflow array when color == P_OVERFLOW
	float friction, restitution, rollingResistance, tangentSpeed;
	float invMassA, invIA, invMassB, invIB;
	Manifold m;
	SimplexCache cache; // chain segment manifolds (contact.h:126)
	// solver set, island and body edge lists (contact.h:44-96)
	int setIndex;
	int islandId, islandPrev, islandNext;
	int edgePrev[2], edgeNext[2]; // edge 0 on bodyA's list, edge 1 on bodyB's
	int isMarked;
} Contact;

// Per-constraint solver data (contact_solver.c:1034-1064 lanes / contact_solver.h)
typedef struct ConstraintPoint
{
	v2 anchorA, anchorB;
	float baseSeparation;
	float relativeVelocity;
	float normalImpulse;
	float tangentImpulse;
	float totalNormalImpulse;
	float normalMass;
	float tangentMass;
} ConstraintPoint;

typedef struct Constraint
{
	int contactId;
	int indexA, indexB; // body ids, -1 for static
	float invMassA, invIA, invMassB, invIB;
	v2 normal;
	float friction, restitution, tangentSpeed, rollingResistance, rollingMass, rollingImpulse;
	float biasRate, massScale, impulseScale; // softness
	ConstraintPoint points[2];
	int pointCount;
} Constraint;

typedef struct Softness
{
	float biasRate, massScale, impulseScale;
} Softness;

enum
{
	P_JOINT_REVOLUTE = 1,
	P_JOINT_WELD = 2,
	P_JOINT_DISTANCE = 3,
	P_JOINT_PRISMATIC = 4,
	P_JOINT_WHEEL = 5,
	P_JOINT_MOTOR = 6,
	P_JOINT_MOUSE = 7,
	P_JOINT_FILTER = 8,
};

typedef struct Joint
{
	int used;
	int generation;
	int type; // P_JOINT_*
	int bodyA, bodyB;
	int color;
	int colorBodies; // bit 0 / 1: body A / B took the colour's bit when coloured
	int overflowIndex;
	int collideConnected;
	int nextA, prevA, nextB, prevB; // body joint lists (joint keys)
	// revolute definition (revolute_joint.c / joint.h:247-278)
	v2 localOriginAnchorA, localOriginAnchorB;
	float referenceAngle, targetAngle;
	float hertz, dampingRatio;
	float lowerAngle, upperAngle;
	float maxMotorTorque, motorSpeed;
	int enableSpring, enableLimit, enableMotor;
	float drawSize;
	float constraintHertz, constraintDampingRatio;
	// solver state
	v2 linearImpulse;
	float springImpulse, motorImpulse, lowerImpulse, upperImpulse;
	// prepared
	int indexA, indexB;
	v2 anchorA, anchorB;
	v2 deltaCenter;
	float deltaAngle;
	float axialMass;
	Softness springSoftness, constraintSoftness;
	float invMassA, invMassB, invIA, invIB;
	// weld (weld_joint.c)
	float linearHertz, linearDampingRatio, angularHertz, angularDampingRatio;
	float angularImpulse;
	Softness linearSoftness, angularSoftness;
	// distance (distance_joint.c)
	float length, minLength, maxLength, maxMotorForce;
	float impulse;
	Softness distanceSoftness;
	// prismatic and wheel (prismatic_joint.c, wheel_joint.c)
	v2 localAxisA, axisA;
	float targetTranslation, lowerTranslation, upperTranslation;
	v2 prismaticImpulse; // perpendicular, angular
	float perpImpulse, perpMass, motorMass;
	// motor and mouse (motor_joint.c, mouse_joint.c)
	v2 linearOffset;
	float angularOffset, maxForce, maxTorque, correctionFactor;
	v2 linearMassCx, linearMassCy;
	float angularMass;
	v2 targetA;
	// solver set and island (joint.h:60-100)
	int setIndex;
	int islandId, islandPrev, islandNext;
	int isMarked;
} Joint;

// growable int array and LIFO id pool (id_pool.c)
typedef struct IntArr
{
	int* data;
	int count, cap;
} IntArr;

typedef struct IdPool
{
	IntArr freeIds;
	int next;
} IdPool;

// solver sets (solver_set.h): 0 static, 1 disabled, 2 awake, 3.. sleeping
enum
{
	SET_STATIC = 0,
	SET_DISABLED = 1,
	SET_AWAKE = 2,
	SET_FIRST_SLEEPING = 3,
};

typedef struct SolverSet
{
	int setIndex; // P_NULL when free
	IntArr bodies, contacts, joints, islands; // ids in set order
} SolverSet;

// island.h:30-60
typedef struct Island
{
	int setIndex, localIndex, islandId;
	int headBody, tailBody, bodyCount;
	int headContact, tailContact, contactCount;
	int headJoint, tailJoint, jointCount;
	int parentIsland;
	int constraintRemoveCount;
} Island;

typedef struct PairSet
{
	uint64_t* keys; // 0 = empty, key+1 stored
	int cap;
	int count;
} PairSet;

typedef struct PChain
{
	int used, generation, bodyId;
	int nextChain;
	int count;
	int* shapeIds;
} PChain;

typedef struct World
{
	int used;
	f2d_world_def def;
	v2 gravity;
	float contactHertz, contactDampingRatio, maxContactPushSpeed, maximumLinearSpeed;
	float restitutionThreshold, hitEventThreshold;
	float contactSpeed, inv_h;
	int enableSleep, enableContinuous, enableWarmStarting;

	Body* bodies;
	int bodyCount, bodyCap;
	int* bodyFree;
	int bodyFreeCount;

	Shape* shapes;
	int shapeCount, shapeCap;
	int* shapeFree;
	int shapeFreeCount;

	Contact* contacts;
	int contactCount, contactCap; // count = id capacity used
	int* contactFree;
	int contactFreeCount;

	Joint* joints;
	int jointCount, jointCap;
	int* jointFree;
	int jointFreeCount;

	// chains (shape.c:339-486): the segment shape ids of each chain
	struct PChain* chains;
	int chainCount, chainCap;
	int* chainFree;
	int chainFreeCount;

	// the reference's three broadphase trees (static, kinematic, dynamic)
	RTree trees[3];
	PairSet pairs;

	// move buffer in deterministic order (shape ids), and a compact copy of
	// the shapes' moved flags (the pair queries test it for every leaf)
	int* moveArray;
	int moveCount, moveCap;
	unsigned char* movedFlag;
	int movedFlagCap;

	// overflow colour order (contact ids / joint ids) as the reference's
	// colour-11 arrays keep them: append on add, swap-remove on remove
	int* overflowContacts;
	int overflowCount, overflowCap;
	int* overflowJoints;
	int overflowJointCount, overflowJointCap;

	// parity plan: contact ids to use for pairs created in the next step
	int* plan;
	int planCount, planCap;

	// scratch
	Constraint* constraints;
	int constraintCap;

	// events of the last step
	int* beginEvents; // pairs shapeA shapeB
	int beginCount, beginCap;
	// the manifold of each begin event (types.h b2ContactBeginTouchEvent):
	// normal, point count, then per point the world point and separation
	float* beginManifolds;
	int beginManifoldCap;
	int* endEvents;
	int endCount, endCap;
	int* hitShapes;
	float* hitData;
	int hitCount, hitCap, hitDataCap;
	int* moveEventBodies;
	float* moveEventXf;
	int moveEventCount, moveEventCap, moveEventXfCap;
	// batched form: independent sub-worlds in one world, each with its own
	// gravity; shapes of different sub-worlds never interact
	int subCount; // 0 = no sub-worlds (one world, world gravity)
	v2 subGravity;
	// static shapes in the static tree's depth-first visiting order (the
	// order continuous collision meets them), rebuilt when that tree changes
	int* staticOrder;
	int staticOrderCount, staticOrderCap, staticOrderDirty;
	int* constraintOrder; // contact id per constraint slot
	int constraintOrderCap;
	int* jointOrder; // graph-colour joints grouped by colour
	int jointOrderCap;

	int stepIndex;
	// the step's tree rebuild runs beside the narrowphase and solver, as the
	// reference's task does (world.c:488-502, solver.c:1824-1830)
	pthread_t treeThread;
	int treeThreadActive;
	int treeThreadsSaved; // OpenMP threads to restore when it is joined

	// islands and solver sets
	Island* islands;
	int islandCap;
	IdPool islandPool;
	SolverSet* sets;
	int setCap;
	IdPool setPool;
	int splitIslandId;
	int* moveEventAsleep; // fellAsleep flag per move event
	int moveEventAsleepCap;
	// sensors (sensor.c): sensor shapes in creation order with their sorted
	// overlaps of the previous and the current step; this step's events as
	// (sensor shape, visitor shape) pairs
	struct PSensor* sensors;
	int sensorCount, sensorCap;
	IntArr sensorBegin, sensorEnd;
	// end events made between steps (destroyed contacts and sensors): the
	// reference reports them with the next step's end events, first
	// (world.c:808-810 double buffer)
	IntArr pendingEnd, pendingSensorEnd;
	// user callbacks (world.c b2World_SetCustomFilterCallback / SetPreSolveCallback)
	orc_custom_filter_fn customFilter;
	void* customFilterContext;
	orc_pre_solve_fn preSolve;
	void* preSolveContext;
} World;

typedef struct PSensor
{
	int shapeId;
	IntArr overlaps1, overlaps2; // visitor shape ids, ascending
} PSensor;
void p_overlap_sensors( World* w ); // psensor.c

// islands and solver sets (pisland.c)
void ia_push( IntArr* a, int v );
int ia_remove_swap( IntArr* a, int index );
void ia_free( IntArr* a );
void p_sets_init( World* w );
void p_sets_free( World* w );
int p_set_body_add( World* w, int setId, int bodyId );
void p_create_island_for_body( World* w, int setId, int bodyId );
void p_contact_edges_link( World* w, int cid );
void p_contact_edges_unlink( World* w, int cid );
void p_link_contact( World* w, int cid );
void p_unlink_contact( World* w, int cid );
void p_link_joint( World* w, int jid, int mergeIslands );
void p_merge_awake_islands( World* w );
void p_split_island( World* w, int baseId );
void p_try_sleep_island( World* w, int islandId );
void p_wake_solver_set( World* w, int setId );
void p_sleep_islands( World* w, const unsigned char* awakeIslandBits, int splitCandidate );
int p_body_awake( const World* w, int bodyId );
void p_static_order( World* w );
void p_finish_tree_rebuild( World* w );
int p_new_sleeping_set( World* w );
void p_set_joint_add( World* w, int setId, int jid );
void p_merge_solver_sets( World* w, int setId1, int setId2 );
void p_unlink_joint( World* w, int jid );
void p_transfer_body( World* w, int targetSet, int bodyId );
void p_transfer_joint( World* w, int targetSet, int jid );
void p_remove_body_from_island( World* w, int bodyId );
void p_set_remove_body( World* w, int bodyId );
void p_set_remove_contact( World* w, int cid );
void p_set_remove_joint( World* w, int jid );
int p_wake_body( World* w, int bodyId );
void p_joint_created( World* w, int jid );
// constraint graph (pworld.c)
void p_add_contact_to_graph( World* w, int cid );
void p_remove_contact_from_graph( World* w, int cid );
void p_add_joint_to_graph( World* w, int jid );
void p_remove_joint_from_graph( World* w, int jid );

// geometry (pgeom.c)
int p_compute_hull( const v2* points, int count, v2* hull );
Polygon p_make_polygon( const v2* hull, int count, float radius );
Polygon p_make_offset_rounded_box( float hx, float hy, v2 center, rot q, float radius );
MassData p_shape_mass( const Shape* s );
box2 p_shape_aabb( const Geometry* g, xform xf );
v2 p_shape_centroid( const Geometry* g );
void p_shape_extent( const Shape* s, v2 localCenter, float* minExtent, float* maxExtent );
float p_shape_radius( const Geometry* g );

// manifolds (pmanifold.c)
Manifold p_collide( const Geometry* a, xform xfA, const Geometry* b, xform xfB, SimplexCache* cache );
int p_manifold_registered( int typeA, int typeB, int* primary );

// distance / time of impact (pdistance.c)
typedef struct ShapeProxy
{
	v2 points[P_MAX_POLY];
	int count;
	float radius;
} ShapeProxy;
typedef struct Sweep
{
	v2 localCenter;
	v2 c1, c2;
	rot q1, q2;
} Sweep;
float p_shape_distance( const ShapeProxy* pa, const ShapeProxy* pb, xform xfA, xform xfB, SimplexCache* cache,
						v2* pointA, v2* pointB, v2* normal );
ShapeProxy p_make_proxy( const v2* pts, int count, float radius );
ShapeProxy p_shape_proxy( const Geometry* g );
float p_time_of_impact( const ShapeProxy* pa, const ShapeProxy* pb, Sweep sa, Sweep sb, float maxFraction, int* state );

// joints (pjoint.c)
Softness p_make_soft( float hertz, float zeta, float h );

// cumulative seconds per step phase: pairs, collide, state changes, solver
// set-up, substeps, restitution + store, finalize + continuous, events
double p_now( void );
extern double g_portPhase[8];
void p_prepare_joint( World* w, Joint* j, float h, float inv_h, Softness jointSoftness );
void p_warm_start_joint( World* w, Joint* j );
void p_solve_joint( World* w, Joint* j, float h, float inv_h, int useBias );
