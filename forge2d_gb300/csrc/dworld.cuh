// Device-resident world state: structure-of-arrays body, shape, contact,
// joint and constraint records in HBM, plus the step's scratch buffers.
//
// Indexing follows the reference's stable ids: bodies by body id, shapes by
// shape id, contacts by contact id (b2Contact array indexed by the contact id
// pool, packages/forge2d/third_party/box2d/src/contact.c:186-240). Static
// bodies keep rows too; the solver treats them as the identity state
// (contact_solver.c:1195-1201 dummy body).
#pragma once

#include "dmath.cuh"

#include <cuda_runtime.h>

// body flags
#define BF_USED 0x1
#define BF_ENABLED 0x2
#define BF_BULLET 0x4
#define BF_FAST_ROT 0x8
#define BF_FIXED_ROT 0x10
#define BF_ENABLE_SLEEP 0x20
#define BF_SPEED_CAPPED 0x40
#define BF_IS_FAST 0x80
#define BF_ENLARGE 0x100
#define BF_ASLEEP 0x200 // in a sleeping solver set
#define BF_TYPE_SHIFT 16 // 2 bits: 0 static 1 kinematic 2 dynamic

// shape flags
#define SF_USED 0x1
#define SF_SENSOR 0x2
#define SF_CONTACT_EVENTS 0x4
#define SF_HIT_EVENTS 0x8
#define SF_PRESOLVE 0x10
#define SF_ENLARGED 0x20
#define SF_MOVED 0x40
#define SF_PROXY 0x80 // has a broadphase proxy
#define SF_SENSOR_EVENTS 0x100 // enableSensorEvents
#define SF_TYPE_SHIFT 16

// shape types (b2ShapeType)
#define ST_CIRCLE 0
#define ST_CAPSULE 1
#define ST_SEGMENT 2
#define ST_POLYGON 3
#define ST_CHAIN 4 // chain segment (one-sided, with ghost vertices)

// contact flags (contact.h:74-93 sim flags plus the b2Contact flags)
#define CF_USED 0x1
#define CF_TOUCHING 0x2 // b2_contactTouchingFlag (graph membership)
#define CF_EVENTS 0x4	// b2_contactEnableContactEvents
#define CF_SIM_TOUCHING 0x10000
#define CF_DISJOINT 0x20000
#define CF_STARTED 0x40000
#define CF_STOPPED 0x80000
#define CF_HIT_EVENT 0x100000
#define CF_PRESOLVE 0x200000
#define CF_INACTIVE 0x400000 // not in the awake set (disabled or sleeping): not collided

// error bits in DScalars::error
#define ERR_CONTACT_CAPACITY 0x1
#define ERR_PAIR_CAPACITY 0x2
#define ERR_BARRIER_TIMEOUT 0x4
#define ERR_PLAN_MISMATCH 0x8
#define ERR_OP_CAPACITY 0x10
#define ERR_COLOR_ROUNDS 0x20
#define ERR_EVENT_CAPACITY 0x40
#define ERR_TREE 0x80

// Shape geometry record: 10 float4 per shape.
//   g[0] = c1.x c1.y c2.x c2.y   (circle centre; capsule/segment ends; polygon centroid)
//   g[1] = radius, count (int bits), localCentroid.x, localCentroid.y
//   g[2..5] polygon vertices, g[6..9] polygon normals
//   chain segment: g[0] = point1 point2, g[2] = ghost1.xy ghost2.xy
#define GEOM_F4 10

// Narrowphase manifold classes (one bucket and one kernel each): circle pairs,
// capsule/segment vs circle, capsule/segment vs capsule, polygon vs circle,
// and the pairs that go through the polygon clipper (or have no manifold).
#define NP_CLASSES 5

// Colouring op outputs: tiles of OPS_TILE ops, four look-back chains
// (freed ids, begin events, end events, overflow ops) after a ticket word.
#define OPS_TILE 1024
#define OPS_SCAN_CHAINS 4
#define OPS_SCAN_WORDS( cap ) ( 1 + OPS_SCAN_CHAINS * ( ( ( cap ) + OPS_TILE - 1 ) / OPS_TILE + 1 ) )

// The tree's leaf order only sets its tightness, never the pairs it finds
// (new pairs are sorted by key), so it is refreshed periodically.
#define ORDER_REBUILD_PERIOD 8

// Per-step scalars kept in device memory so that no launch needs a host
// round trip.
struct DScalars
{
	int contactIdCount; // high-water mark of the contact id pool
	int contactFreeCount;
	int newPairCount;
	int opCount;
	int touchingCount;
	int colorCount[F2D_COLORS];
	int colorStart[F2D_COLORS + 1];
	int overflowCount;
	int overflowJointCount;
	int fastCount;
	int beginCount, endCount, hitCount, moveCount;
	int error;
	int colorRounds;
	unsigned barrierCount;
	unsigned ptBarrier; // the tree rebuild's grid barrier (it runs beside other kernels)
	unsigned barrierGen;
	int planCount;
	int awakeCount;
	int treeLeafCount;
	float contactSpeed;
	int stepIndex;
	// leaf order of the broadphase tree: re-sorted when forced (proxy set or
	// shape rows changed) or every ORDER_REBUILD_PERIOD steps, reused between
	int rebuildOrder;
	int forceRebuild;
	int orderAge;
	int orderPeriod; // steps between re-sorts (0: ORDER_REBUILD_PERIOD)
	int newPointCount; // new manifold points listed by the prepare stage (learned warm start)
	int sampleCount;   // training samples recorded so far
	int npCount[8];	   // narrowphase: live overlapping contacts per manifold class
	int pendingOps;	   // colouring: ops left after the first round
	int overflowOps;   // colouring: ops that add to / remove from the overflow colour
	int sensorCur, sensorPrev;	   // sensor overlaps this step / last step
	int sensorBegin, sensorEnd;	   // sensor events of this step
	int cbList, cbReject;		   // user callbacks: listed candidates, rejected keys
	// the reference's broadphase trees (static, kinematic, dynamic) and the
	// move array: root node, proxies; proxies in the move array, proxies the
	// host buffered since the last step
	int treeRoot[3];
	int treeProxies[3];
	int moveArrayCount;
	int hostMoveCount;
	// partial rebuild of one tree: active, gathered nodes, large segments
	// per level (two levels in flight), small segments
	int rbActive, rbCount, rbLarge[2], rbSmall, rbRefresh;
	// creation stamp of the next new contact (the bodies' contact lists are
	// newest first); non-static bodies in the awake set (worlds without
	// island records); destroy calls: collected contacts, end events
	int solveBarriers; // grid barriers the last grid-wide solver launch passed
	unsigned long long stampBase;
	int awakeOrderCount;
	int apiCount, apiEndCount;
};

// node flags of the broadphase trees (dynamic_tree.c b2TreeNodeFlags)
#define PT_ALLOCATED 1
#define PT_ENLARGED 2
#define PT_LEAF 4

// ---------------------------------------------------------------------------
// The reference's broadphase trees (dynamic_tree.c), one per body type, kept
// node for node: ids, topology, boxes, heights, categories and flags (bits
// PT_ALLOCATED, PT_ENLARGED, PT_LEAF of htree.h). The host inserts and
// removes proxies (htree.cpp); the device enlarges proxies and rebuilds the
// enlarged part every step (proxytree.cu). `leaves` counts the leaves of a
// subtree; `rank` is a leaf's left-to-right position and `rankShape` its
// inverse, from which the order of new contacts is made.
// ---------------------------------------------------------------------------
struct DProxyTree
{
	int cap;
	int* child1;
	int* child2;
	int* parent;
	int* height;
	int* flags;
	int* shape;
	int* leaves;
	float4* box; // lower.x lower.y upper.x upper.y
	unsigned long long* cat;
	int* rank;
	int* rankShape;
};

// Scratch of the partial rebuild (sized by the largest tree capacity).
// Segments are (start, end, child1 edges above, -) ranges of the gathered
// nodes; a chunk is PT_CHUNK consecutive gathered nodes of one segment.
struct DRebuild
{
	int cap, segCap, chunkCap;
	int* doomed;   // internal node being rebuilt
	int* cnt;	   // arrival counters of the bottom-up passes
	int* rlc;	   // gathered nodes below a doomed node
	int* gIdx;	   // gathered nodes, left to right, then partitioned
	float2* gCen;  // their box centres
	int* freed;	   // doomed nodes in pre-order (the reference's free order)
	int* bl;	   // per segment: positions of left-side nodes that belong right
	int* br;	   // and of right-side nodes that belong left, from the end
	int4* segA;
	int4* segB;
	int4* segSmall;
	int* chunkBase; // per large segment: first chunk (and the total at [count])
	int* chunkStat; // per chunk: below pivot, bad left, bad right, left offset, right offset
	int* segBounds; // per large segment: centre bounds as ordered ints
	int* segBelow;	// per large segment: centres below the pivot
	int* pairBase;	// per large segment: first swap pair
	int* rfStart;	// children of the large levels the bottom-up pass starts from
};

// ---------------------------------------------------------------------------
// Islands and solver sets (island.h, solver_set.h), kept on the device in
// worlds with sleeping enabled and updated by single-thread kernels in the
// reference's serial order (island.cu). Set ids: 0 static, 1 disabled,
// 2 awake, 3.. sleeping. A sleeping set's members are kept as append-only
// lists (its array order); the awake set's bodies and islands as arrays with
// swap-remove, as the reference keeps them.
// ---------------------------------------------------------------------------
#define SET_STATIC 0
#define SET_DISABLED 1
#define SET_AWAKE 2
#define SET_FIRST_SLEEPING 3

struct DIsland
{
	int setIndex, localIndex;
	int headBody, tailBody, bodyCount;
	int headContact, tailContact, contactCount;
	int headJoint, tailJoint, jointCount;
	int parent, removeCount;
	int setNext; // next island of the same sleeping set
};

struct DSet
{
	int used;
	int headBody, tailBody, bodyCount;
	int headContact, tailContact, contactCount;
	int headJoint, tailJoint, jointCount;
	int headIsland, tailIsland, islandCount;
};

struct DIslands
{
	int bodyCap, contactCap, jointCap, islandCap, setCap;
	// bodies
	int* bSet;
	int* bLocal; // index in the awake body array
	int* bIsland;
	int* bIslandPrev;
	int* bIslandNext;
	int* bHeadContact; // contact edge list: (contactId << 1) | edge
	int* bSetNext;
	int* bMark;
	int* bMoveIndex; // this step's move-event slot, -1 when none
	// contacts
	int* cSet;
	int* cIsland;
	int* cIslandPrev;
	int* cIslandNext;
	int* cSetNext;
	int* cMark;
	int4* cEdge; // prev0 next0 prev1 next1 (edge 0 on bodyA's list)
	// joints
	int* jSet;
	int* jIsland;
	int* jIslandPrev;
	int* jIslandNext;
	int* jSetNext;
	int* jMark;
	int* jOverflowIndex;
	// islands, sets, pools
	DIsland* islands;
	int* islandFree;
	DSet* sets;
	int* setFree;
	int* awakeBodies;
	int* awakeIslands;
	unsigned char* islandBits;
	int* stack;	   // split scratch, bodyCap
	int* seeds;	   // split scratch, bodyCap
	int* order;	   // new-contact creation order, contactCap
	int* flag;		   // per awake island: scan input (bodyCap)
	int* pos;		   // scan output (bodyCap)
	int* list;		   // compacted island ids (bodyCap)
	int listCount;
	unsigned long long candKey; // split candidate: sleep-time bits << 32 | ~awake index
	int* moveBody;	   // move events of the step in awake order
	int* moveAsleep;   // fellAsleep per move event
	int* log;		   // creation log: (kind << 30) | id, kind 0 body, 1 joint
	int logCap;
	int logCount;
	int bodyKnown; // bodies below this id have set and island records
	int islandFreeCount, islandNext;
	int setFreeCount, setNext;
	int awakeBodyCount, awakeIslandCount;
	int splitIslandId;
	int moveCount;
	int splitCandidate;
	int error;
	// state changes: 1 when a contact that began touching wakes a sleeping
	// set (the step's changes then run serially), and the per-contact marks
	// of the parallel unlink (bit 0 island list, bit 1 body edge lists)
	int serialOps;
	unsigned char* cRemoved;
	// new contacts' body edges sorted by (body, creation rank): keys and
	// their capacity (2 x the new-pair capacity)
	unsigned long long *ncKeys, *ncKeysAlt;
	int ncCap, ncCount;
	int linkCount; // contacts that began touching this step (parallel links)
};

// Solver view of one body: velocity and the substep position/rotation
// deltas (b2BodyState, body.h:101-113).
struct BState
{
	float vx, vy, w;
	float dpx, dpy, dqc, dqs;
};

struct DWorld
{
	// capacities
	int bodyCap, shapeCap, contactCap, jointCap;
	int pairCap;  // new-pair buffer capacity per step
	int pairKeyBits; // sort key of a new pair: (min shape id << pairKeyBits) | max shape id
	int opCap;	  // state-change op capacity per step
	int hashCap;  // pair-set hash capacity (power of two)
	int eventCap; // per-step event buffer capacity

	// host-known counts (creation path)
	int bodyCount, shapeCount, jointCount;

	// world constants
	fv2 gravity;
	float restitutionThreshold, hitEventThreshold;
	float contactHertz, contactDampingRatio, maxContactPushSpeed, maxLinearSpeed;
	float jointHertz, jointDampingRatio;
	int enableSleep, enableContinuous, enableWarmStarting;
	int subCount; // batched form: independent sub-worlds (0 = one world)

	// learned warm start: bit 0 records (features, final impulses) of new
	// manifold points as training samples, bit 1 predicts their initial
	// impulses with model mlpModel
	int learnMode;
	int mlpModel;
	int newPointCap;
	int2* newPoint; // (constraint slot, point index)
	float* newFeat; // 12 features per new point
	int sampleCap;
	float* samples; // 14 floats per sample

	// ---------------- bodies (by body id) ----------------
	float4* xf;			// p.x p.y q.c q.s
	float4* vel;		// v.x v.y w flags-pad      (b2BodyState bytes 0..15)
	float4* delta;		// dp.x dp.y dq.c dq.s      (b2BodyState bytes 16..31)
	float2* center;		// world centre of mass
	float4* sweep0;		// center0.x center0.y rotation0.c rotation0.s
	float2* localCenter;
	float4* massv;		// invMass invInertia minExtent maxExtent
	float4* damp;		// linearDamping angularDamping gravityScale sleepThreshold
	float4* force;		// force.x force.y torque sleepTime
	float2* bodyGravity; // gravity of the body's sub-world (batched form, subCount > 0)
	int* bflags;
	int* headShape;
	int* headJoint; // joint key list: (jointId << 1) | edge
	int* jointCountB;
	unsigned* colorMask; // bit c: body holds a graph constraint of colour c < 11
	int* colorLock;		 // scratch for the colouring rounds

	// ---------------- shapes (by shape id) ----------------
	float4* geom; // GEOM_F4 per shape
	float4* aabb;
	float4* fat;
	float4* mat; // friction restitution rollingResistance tangentSpeed
	unsigned long long* cat;
	unsigned long long* mask;
	int* group;
	int* shapeBody;
	int* sflags;
	int* proxyKey;
	int* nextShape;
	int* shapeSub; // sub-world of the owning body (batched form)

	// ---------------- contacts (by contact id) ----------------
	int2* cshape; // shapeA shapeB
	int2* cbody;  // bodyA bodyB
	int* cflags;
	int* ccolor;
	int* coverflowIndex;
	float4* cmat;  // friction restitution rollingResistance tangentSpeed
	float4* cmass; // invMassA invIA invMassB invIB
	float4* mnorm; // normal.x normal.y rollingImpulse pointCount(bits)
	int2* csimplex; // GJK cache of chain segment manifolds: count | indexA[0..2] << 8.., indexB[0..2]
	float4* mpA;   // [2*id+k] anchorA.xy anchorB.xy
	float4* mpB;   // [2*id+k] point.xy separation id(bits, bit16 = persisted)
	float4* mpI;   // [2*id+k] normalImpulse tangentImpulse totalNormalImpulse normalVelocity
	int* contactFree; // LIFO free id stack (id_pool.c:19-38)
	unsigned long long* pairHash; // open-addressing set of live pair keys (key+1)

	// ---------------- broadphase scratch ----------------
	unsigned* mortonKeys;
	unsigned* mortonKeysAlt;
	int* leafShape;
	int* leafShapeAlt;
	int* nodeLeft;	 // internal node children; leaves encoded as ~leafIndex
	int* nodeRight;
	int* nodeParent; // [internal nodes, then leaves]
	float4* nodeBox;
	int* nodeVisit;
	unsigned* sortHist; // radix sort histograms
	unsigned long long* pairKeys;
	unsigned long long* pairKeysAlt;
	int* pairVal;
	int* pairValAlt;
	int* planIds; // parity plan: contact ids by ascending pair key
	unsigned long long* planKeys;
	int* newPairId; // parity mode: the contact id given to each new pair (creation order)

	// ---------------- state-change ops ----------------
	int* opContact; // contact id
	int* opKind;	// 0 destroy, 1 begin, 2 end
	int* opColor;	// colour result / colour removed
	int* opDone;
	int2* opBodies; // solver body indices of the op's contact (-1 static)
	unsigned long long* opScan; // look-back state of the op output scans

	// ---------------- constraints (by slot, grouped by colour) ----------------
	int* slotContact;
	int* overflowList; // contact ids in overflow-array order
	int2* kIndex;	   // indexA indexB (-1 static)
	float4* kMass;	   // invMassA invIA invMassB invIB
	float4* kNormal;   // normal.x normal.y friction tangentSpeed
	float4* kMisc;	   // restitution rollingResistance rollingMass rollingImpulse
	float4* kSoft;	   // biasRate massScale impulseScale pointCount(bits)
	float4* kAnch1;	   // anchorA1.xy anchorB1.xy
	float4* kAnch2;	   // anchorA2.xy anchorB2.xy
	float4* kP1;	   // baseSeparation normalMass tangentMass relativeVelocity (point 1)
	float4* kP2;	   // same, point 2
	float4* kImp;	   // normalImpulse1 normalImpulse2 tangentImpulse1 tangentImpulse2
	float2* kTot;	   // totalNormalImpulse1 totalNormalImpulse2

	// ---------------- joints (by joint id) ----------------
	int2* jbody;
	int* jflags; // used, enableSpring, enableLimit, enableMotor, collideConnected; type in bits 8-11
	int* jcolor;
	int* jcolorSet; // bit 0 / 1: body A / B took the colour's bit when the joint was coloured
	int* jnext;	 // [2*id+edge] next joint key in the body list
	// definition, impulse and prepared rows; the revolute layout is given,
	// the other types' layouts sit beside their solvers
	float4* jdef0; // localOriginAnchorA.xy localOriginAnchorB.xy
	float4* jdef1; // referenceAngle targetAngle hertz dampingRatio
	float4* jdef2; // lowerAngle upperAngle maxMotorTorque motorSpeed
	float4* jdef3; // type-specific (prismatic spring hertz, damping ratio)
	float4* jimp;  // linearImpulse.xy springImpulse motorImpulse
	float2* jimp2; // lowerImpulse upperImpulse
	float4* jprep0; // anchorA.xy anchorB.xy
	float4* jprep1; // deltaCenter.xy deltaAngle axialMass
	float4* jprep2; // springSoftness biasRate massScale impulseScale, pad
	float4* jprep3; // type-specific (joint axis, 2x2 effective mass)
	float4* jprepM; // invMassA invIA invMassB invIB
	int2* jindex;	// solver body indices
	int* overflowJoints;
	// overflow levels (solver scratch): body owner per level round, level
	// per overflow constraint, constraints in level order beyond the
	// shared-memory list
	int* npBucket; // narrowphase: contact ids by manifold class, NP_CLASSES x contactCap
	DIslands* isl;  // islands and solver sets (sleeping worlds only, else null)
	int* islFlag;	// device copies of isl->flag and isl->pos (scan arguments)
	int* islPos;
	unsigned long long *islNcKeys, *islNcKeysAlt; // copies of isl->ncKeys, ncKeysAlt (sort arguments)
	int* ovfOwner; // bodyCap
	int* ovfLevel; // contactCap + jointCap
	int* ovfOrder; // contactCap + jointCap
	int* pendingJointOps; // joint ids whose colour must be assigned at next step
	int pendingJointCount;

	// ---------------- finalize / events ----------------
	int* fastBodies;
	int* beginEv; // [2*i] shapeA shapeB
	float* beginEvF; // [9*i] manifold: normal.xy pointCount, per point point.xy separation
	int* endEv;
	int* hitEvI;
	float* hitEvF; // [5*i] point normal approachSpeed
	int* moveEvBody;
	float4* moveEvXf;
	int* staticShapes; // compact list of static proxies (CCD candidates)
	// sensors (sensor.c): sensor shapes in creation order; sorted overlap keys
	// (sensor index << 32 | visitor shape) of this step and the last; events
	int* sensorShapes;
	int sensorCount, sensorPairCap;
	unsigned long long *sensorKeys, *sensorKeysAlt, *sensorPrevKeys;
	int2 *sensorBeginEv, *sensorEndEv; // (sensor shape, visitor shape)
	// user callbacks (custom filter, pre-solve), evaluated on the host
	// between launches: candidates the device lists for the host
	// (continuous pairs static << 32 | fast; pre-solve contact ids with
	// their manifolds), and the sorted keys the host rejected
	int callbacks;	 // bit 0 custom filter, bit 1 pre-solve
	int cbCap;
	unsigned long long* cbList;
	float* cbManifold; // 22 per listed pre-solve contact: f2d_manifold_view, shape A, shape B
	unsigned long long* cbReject;
	int staticCount;

	// the reference's broadphase trees and the move array (proxytree.cu)
	DProxyTree pt[3];
	int ptProxies[3]; // proxies per tree as of the last upload (host count)
	DRebuild rb;
	int* shapeMove; // per shape: position in the move array
	int* moveShape; // move array: shape ids
	int* hostMoves; // shapes the host buffered since the last step, in call order

	// destroy path: creation stamp per contact, the awake set's body order
	// (worlds without island records), end events of destroyed contacts
	unsigned long long* cstamp;
	int* awakeOrder;
	int* apiEndEv; // [2*i] shapeA shapeB

	DScalars* sc;
	int* sortTemp;
};

#ifdef __CUDACC__
// Left-to-right position of a leaf in one of the reference's trees: the
// leaves of every child1 subtree passed on the way up from the leaf (a
// depth-first query visits overlapping leaves in descending position)
__device__ __forceinline__ int tree_leaf_rank( const DProxyTree& T, int leaf )
{
	int r = 0, c = leaf;
	for ( int guard = 0; guard < ( 1 << 16 ); ++guard )
	{
		int p = T.parent[c];
		if ( p < 0 || p >= T.cap )
			break;
		if ( T.child2[p] == c )
			r += T.leaves[T.child1[p]];
		c = p;
	}
	return r;
}
#endif

__host__ __device__ __forceinline__ int body_type( int f )
{
	return ( f >> BF_TYPE_SHIFT ) & 3;
}
__host__ __device__ __forceinline__ int shape_type( int f )
{
	return ( f >> SF_TYPE_SHIFT ) & 7;
}
