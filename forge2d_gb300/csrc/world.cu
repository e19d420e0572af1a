// Host side of the GPU world: the C ABI of include/forge2d_gb300.h, the
// creation path, device allocation and uploads, and the step driver.
//
// Creation follows Box2D v3.1.1 (packages/forge2d/third_party/box2d/src/
// body.c:177-330, shape.c:36-180, joint.c:146-330, id_pool.c:19-38) on host
// mirrors of the device rows; rows created since the last step are uploaded
// as one contiguous range per array before the step. The step itself is a
// fixed sequence of launches whose sizes come from device-resident counts,
// captured once into a CUDA graph and replayed while the world's capacities
// and step parameters stay the same.
#include "../../include/forge2d_gb300.h"
#include "dscan.cuh"
#include "dsort.cuh"
#include "dworld.cuh"
#include "hgeom.h"
#include "htree.h"
#include "joint.cuh"
#include "kernels.cuh"

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

void launch_reset_counters( DWorld& w, cudaStream_t st );


#define MAX_WORLDS 128

struct HostWorld
{
	bool used = false;
	uint16_t generation = 0;
	int index = 0;
	DWorld d;
	StepScratch s;
	cudaStream_t stream = nullptr;
	cudaEvent_t evStart = nullptr, evStop = nullptr;
	// the tree rebuild's stream and its fork / join events
	cudaStream_t stream2 = nullptr;
	cudaEvent_t evFork = nullptr, evJoin = nullptr;
	int* hostError = nullptr; // pinned
	int statusAccum = 0;
	bool stepped = false;
	float lastStepMs = 0.0f;
	int lastLaunches = 0;

	// phase timing (profiling mode: no graph, events between phases)
	bool profiling = false;
	cudaEvent_t ph[9] = {}; // [7], [8]: the tree rebuild on its own stream

	// graph replay
	cudaGraphExec_t graphExec = nullptr;
	float graphDt = 0.0f;
	int graphSubSteps = 0;
	int graphKernelNodes = 0;
	bool graphDirty = true;

	// ---- host mirrors (same layout as the device rows) ----
	std::vector<float4> xf, vel, delta, sweep0, massv, damp, force;
	std::vector<float2> bgrav;
	std::vector<int> bsub;
	std::vector<float2> center, localCenter;
	std::vector<int> bflags, headShape, headJoint, jointCountB;
	std::vector<uint16_t> bgen;
	std::vector<float> bmass, binertia;
	std::vector<int> bodyFree;
	std::vector<std::string> bname; // b2Body_SetName (host only)
	int bodyCount = 0, bodyUploaded = 0;
	std::vector<int> bodyDirty;
	std::vector<uint8_t> bodyIsDirty; // host row newer than the device row

	std::vector<float4> geom, aabb, fat, mat;
	std::vector<unsigned long long> cat, mask;
	std::vector<int> group, shapeBody, sflags, proxyKey, nextShape, ssub;
	std::vector<float> density;
	std::vector<uint16_t> sgen;
	std::vector<HShapeGeom> hgeomv;
	std::vector<int> shapeFree;
	int shapeCount = 0, shapeUploaded = 0;
	std::vector<int> shapeDirty;
	// the reference's broadphase trees (static, kinematic, dynamic): the
	// host inserts and removes; the device enlarges and rebuilds the
	// kinematic and dynamic trees every step, so those are read back before
	// a host edit (treeStale) and sent after it (treeDirty)
	HTree trees[3];
	bool treeDirty[3] = { true, true, true };
	bool treeStale[3] = { false, false, false };
	// proxies buffered for the next step's pair search since the last step
	// (creation, transforms), in call order, each once
	std::vector<int> hostMoves;
	std::vector<uint8_t> hostMoved;
	std::vector<int> staticShapes; // static shapes in the static tree's query order
	int treeScalars[6] = {};	   // staging of the trees' roots and proxy counts
	int hostMoveCount = 0;		   // staging of the buffered proxy count
	std::vector<int> sensorShapes; // sensor shapes in creation order (sensor.c)
	float invH = 0.0f; // inverse substep of the last step (world.c:745-755)
	f2d_custom_filter_fn customFilter = nullptr;
	void* customFilterContext = nullptr;
	f2d_pre_solve_fn preSolve = nullptr;
	void* preSolveContext = nullptr;
	bool sensorsDirty = false;
	// chains: segment shape ids and generation per chain id (LIFO id reuse)
	std::vector<std::vector<int>> chainSegments;
	std::vector<uint16_t> chainGen;
	std::vector<int> chainFree;
	// chains per body (the reference's body chain list, newest first)
	std::vector<int> chainBody, chainNext, headChain;
	bool staticDirty = false;
	// the awake set's non-static bodies in the reference's array order
	// (appended at creation, swap-removed at destruction), for worlds without
	// island records; awakeSlot is a body's position, -1 when absent
	std::vector<int> awakeOrder, awakeSlot;
	bool awakeOrderDirty = true;
	int awakeOrderCount = 0; // staging of the device count
	// end events of contacts and sensors destroyed between steps (four ints
	// per event, ids packed at destruction): `Next` collects them, the next
	// step reports them ahead of its own (`Prefix`), as the reference's
	// double-buffered end event arrays do (world.c:808-810)
	std::vector<int32_t> endNext, endPrefix, sensorEndNext, sensorEndPrefix;
	// a zero time step cleared the step events (world.c:717-725)
	bool eventsCleared = false;

	std::vector<int2> jbody;
	std::vector<int> jflags, jcolor, jnext;
	std::vector<float4> jdef0, jdef1, jdef2, jdef3;
	std::vector<int> jointDirty; // uploaded joints whose definition rows changed on the host
	std::vector<uint8_t> jointIsDirty;
	std::vector<uint16_t> jgen;
	int jointCount = 0, jointUploaded = 0;
	std::vector<int> pendingJoints;
	std::vector<int> jointFree; // LIFO id pool (id_pool.c)
	std::vector<int> jointRows; // reused joint ids whose whole rows go up at the next upload

	// islands and solver sets (worlds with sleeping enabled): host copy of the
	// device record's pointers and capacities, the device record, and the
	// creation log of bodies and joints since the last upload
	bool islOn = false;
	DIslands islHost = {};
	DIslands* islDev = nullptr;
	std::vector<int> islLog;
	int islLogCount = 0;
	bool islBodiesUploaded = false;

	// the broadphase must re-sort its leaf order at the next step
	bool forceRebuild = true;

	// batched form: gravity of the sub-world bodies are created into
	float2 subGravity = { 0.0f, 0.0f };

	// autotuner choice of the tree's leaf-order period (0: default)
	int orderPeriod = 0;

	// solve on the grid-wide cooperative kernel even when the world fits a
	// thread-block cluster (F2D_NO_CLUSTER_SOLVER set at world creation)
	bool gridSolverOnly = false;

	// state of the host mirror of device-changed body rows (MIRROR_*)
	int bodyMirror = 0;

	// device staging of the bulk body reader (12 floats per body)
	float* packedBodies = nullptr;
	int packedCap = 0;

	// plan (parity mode)
	std::vector<unsigned long long> planKeys;
	std::vector<int> planIds;
	bool planPending = false;
};

static HostWorld* s_worlds[MAX_WORLDS];

static int ceil_pow2( int v )
{
	int p = 1;
	while ( p < v )
		p <<= 1;
	return p;
}

template <typename T> static void dgrow( T*& p, size_t oldN, size_t newN )
{
	T* q = nullptr;
	cudaMalloc( (void**)&q, sizeof( T ) * ( newN > 0 ? newN : 1 ) );
	cudaMemset( q, 0, sizeof( T ) * ( newN > 0 ? newN : 1 ) );
	if ( p && oldN > 0 )
		cudaMemcpy( q, p, sizeof( T ) * std::min( oldN, newN ), cudaMemcpyDeviceToDevice );
	if ( p )
		cudaFree( p );
	p = q;
}

template <typename T> static void dfree( T*& p )
{
	if ( p )
		cudaFree( p );
	p = nullptr;
}

// ---------------------------------------------------------------------------
// capacities
// ---------------------------------------------------------------------------
static void alloc_scratch( HostWorld* W )
{
	DWorld& d = W->d;
	StepScratch& s = W->s;
	dfree( s.tmpA );
	dfree( s.tmpB );
	dfree( s.scanTmp );
	dfree( s.bounds );
	int m = std::max( std::max( d.shapeCap, d.contactCap ), std::max( d.bodyCap, d.pairCap ) );
	size_t tmpN = 2 * (size_t)m + 64;
	dgrow( s.tmpA, 0, tmpN );
	dgrow( s.tmpB, 0, tmpN + d.jointCap + 64 );
	int sortBlocks = ( std::max( d.pairCap, d.shapeCap ) + SORT_TILE - 1 ) / SORT_TILE + 1;
	int scanN = std::max( 256 * sortBlocks, m );
	dgrow( s.scanTmp, 0, (size_t)( scanN + SCAN_TILE - 1 ) / SCAN_TILE + 64 );
	dfree( d.sortHist );
	dgrow( d.sortHist, 0, std::max( (size_t)256 * sortBlocks + 256, (size_t)256 * CSORT_MAX_BLOCKS + 256 ) );
	dfree( s.scanState );
	dgrow( s.scanState, 0, (size_t)( m + LB_TILE - 1 ) / LB_TILE + 8 );
	s.sortBlocks32 = sort_coop_blocks<unsigned>();
	s.sortBlocks64 = sort_coop_blocks<unsigned long long>();
	s.boundsBlocks = 64;
	dgrow( s.bounds, 0, (size_t)s.boundsBlocks );
	int bits = 1;
	while ( ( 1 << bits ) < d.shapeCap )
		bits += 1;
	s.shapeIdBits = bits;
	d.pairKeyBits = bits;
	dfree( d.ovfOwner );
	dfree( d.ovfLevel );
	dfree( d.ovfOrder );
	dgrow( d.ovfOwner, 0, (size_t)d.bodyCap );
	dgrow( d.ovfLevel, 0, (size_t)d.contactCap + d.jointCap );
	dgrow( d.ovfOrder, 0, (size_t)d.contactCap + d.jointCap );
	s.solverThreads = 512;
	s.solverBlocks = solver_max_blocks( 512 );
	s.solverBlocks256 = solver_max_blocks( 256 );
	s.clusterCapacity = W->gridSolverOnly ? 0 : solver_cluster_capacity();
	s.ptBlocks = pt_large_blocks();
}

static void grow_bodies( HostWorld* W, int cap )
{
	DWorld& d = W->d;
	size_t o = d.bodyCap;
	dgrow( d.xf, o, cap );
	dgrow( d.vel, o, cap );
	dgrow( d.delta, o, cap );
	dgrow( d.center, o, cap );
	dgrow( d.sweep0, o, cap );
	dgrow( d.localCenter, o, cap );
	dgrow( d.massv, o, cap );
	dgrow( d.damp, o, cap );
	dgrow( d.bodyGravity, o, cap );
	dgrow( d.force, o, cap );
	dgrow( d.bflags, o, cap );
	dgrow( d.headShape, o, cap );
	dgrow( d.headJoint, o, cap );
	dgrow( d.jointCountB, o, cap );
	dgrow( d.colorMask, o, cap );
	dgrow( d.colorLock, o, cap );
	dgrow( d.fastBodies, o, cap );
	dgrow( d.moveEvXf, o, cap );
	dgrow( d.awakeOrder, o, cap );
	d.bodyCap = cap;
}

static void grow_contacts( HostWorld* W, int cap )
{
	DWorld& d = W->d;
	size_t o = d.contactCap;
	dgrow( d.cshape, o, cap );
	dgrow( d.cbody, o, cap );
	dgrow( d.cflags, o, cap );
	dgrow( d.ccolor, o, cap );
	dgrow( d.coverflowIndex, o, cap );
	dgrow( d.cmat, o, cap );
	dgrow( d.cmass, o, cap );
	dgrow( d.mnorm, o, cap );
	dgrow( d.csimplex, o, cap );
	dgrow( d.mpA, 2 * o, 2 * (size_t)cap );
	dgrow( d.mpB, 2 * o, 2 * (size_t)cap );
	dgrow( d.mpI, 2 * o, 2 * (size_t)cap );
	dgrow( d.contactFree, o, cap );
	dgrow( d.cstamp, o, cap );
	dgrow( d.apiEndEv, 0, 2 * (size_t)cap );
	// step scratch sized by contacts (content not preserved)
	dgrow( d.opContact, 0, cap );
	dgrow( d.opKind, 0, cap );
	dgrow( d.opColor, 0, cap );
	dgrow( d.opDone, 0, cap );
	dgrow( d.opBodies, 0, cap );
	dgrow( d.opScan, 0, (size_t)OPS_SCAN_WORDS( cap ) );
	dgrow( d.slotContact, 0, cap );
	dgrow( d.overflowList, o, cap );
	dgrow( d.npBucket, 0, (size_t)NP_CLASSES * cap );
	dgrow( d.kIndex, 0, cap );
	dgrow( d.kMass, 0, cap );
	dgrow( d.kNormal, 0, cap );
	dgrow( d.kMisc, 0, cap );
	dgrow( d.kSoft, 0, cap );
	dgrow( d.kAnch1, 0, cap );
	dgrow( d.kAnch2, 0, cap );
	dgrow( d.kP1, 0, cap );
	dgrow( d.kP2, 0, cap );
	dgrow( d.kImp, 0, cap );
	dgrow( d.kTot, 0, cap );
	dgrow( d.beginEv, 0, 2 * (size_t)cap );
	dgrow( d.beginEvF, 0, 9 * (size_t)cap );
	dgrow( d.endEv, 0, 2 * (size_t)cap );
	dgrow( d.hitEvI, 0, 2 * (size_t)cap );
	dgrow( d.hitEvF, 0, 5 * (size_t)cap );
	d.contactCap = cap;
	d.opCap = cap;
	d.eventCap = cap;
	int hcap = ceil_pow2( 2 * cap );
	dfree( d.pairHash );
	dgrow( d.pairHash, 0, hcap );
	d.hashCap = hcap;
}

static void grow_shapes( HostWorld* W, int cap )
{
	DWorld& d = W->d;
	size_t o = d.shapeCap;
	dgrow( d.geom, o * GEOM_F4, (size_t)cap * GEOM_F4 );
	dgrow( d.aabb, o, cap );
	dgrow( d.fat, o, cap );
	dgrow( d.mat, o, cap );
	dgrow( d.cat, o, cap );
	dgrow( d.mask, o, cap );
	dgrow( d.group, o, cap );
	dgrow( d.shapeBody, o, cap );
	dgrow( d.shapeSub, o, cap );
	dgrow( d.sflags, o, cap );
	dgrow( d.proxyKey, o, cap );
	dgrow( d.nextShape, o, cap );
	dgrow( d.staticShapes, 0, cap );
	dgrow( d.shapeMove, o, cap );
	dgrow( d.moveShape, 0, cap );
	dgrow( d.hostMoves, 0, cap );
	// broadphase scratch
	dgrow( d.mortonKeys, 0, cap );
	dgrow( d.mortonKeysAlt, 0, cap );
	dgrow( d.leafShape, 0, cap );
	dgrow( d.leafShapeAlt, 0, cap );
	dgrow( d.nodeLeft, 0, cap );
	dgrow( d.nodeRight, 0, cap );
	dgrow( d.nodeParent, 0, 2 * (size_t)cap );
	dgrow( d.nodeBox, 0, 2 * (size_t)cap );
	dgrow( d.nodeVisit, 0, cap );
	d.shapeCap = cap;
	int pc = std::max( 65536, 4 * cap );
	dgrow( d.pairKeys, 0, pc );
	dgrow( d.pairKeysAlt, 0, pc );
	dgrow( d.pairVal, 0, pc );
	dgrow( d.pairValAlt, 0, pc );
	dgrow( d.planKeys, 0, pc );
	dgrow( d.planIds, 0, pc );
	dgrow( d.newPairId, 0, pc );
	d.pairCap = pc;
	if ( d.contactCap < 8 * cap )
		grow_contacts( W, 8 * cap );
}

static void grow_joints( HostWorld* W, int cap )
{
	DWorld& d = W->d;
	size_t o = d.jointCap;
	dgrow( d.jbody, o, cap );
	dgrow( d.jflags, o, cap );
	dgrow( d.jcolor, o, cap );
	dgrow( d.jcolorSet, o, cap );
	dgrow( d.jnext, 2 * o, 2 * (size_t)cap );
	dgrow( d.jdef0, o, cap );
	dgrow( d.jdef1, o, cap );
	dgrow( d.jdef2, o, cap );
	dgrow( d.jdef3, o, cap );
	dgrow( d.jimp, o, cap );
	dgrow( d.jimp2, o, cap );
	dgrow( d.jprep0, 0, cap );
	dgrow( d.jprep1, 0, cap );
	dgrow( d.jprep2, 0, 2 * (size_t)cap );
	dgrow( d.jprep3, 0, cap );
	dgrow( d.jprepM, 0, cap );
	dgrow( d.jindex, 0, cap );
	dgrow( d.overflowJoints, o, cap );
	dgrow( d.pendingJointOps, 0, cap );
	d.jointCap = cap;
}

// Island arrays follow the body, contact and joint capacities; contents are
// kept across growth (the device record's scalars are read back first).
static void isl_ensure( HostWorld* W )
{
	if ( !W->islOn )
		return;
	DWorld& d = W->d;
	DIslands& h = W->islHost;
	bool fresh = W->islDev == nullptr;
	if ( !fresh && h.bodyCap == d.bodyCap && h.contactCap == d.contactCap && h.jointCap == d.jointCap &&
		 h.logCap >= d.bodyCap + d.jointCap && h.ncCap >= 2 * d.pairCap )
		return;
	cudaStreamSynchronize( W->stream );
	if ( fresh )
	{
		memset( &h, 0, sizeof( h ) );
		h.setNext = SET_FIRST_SLEEPING;
		h.splitIslandId = -1;
		cudaMalloc( (void**)&W->islDev, sizeof( DIslands ) );
	}
	else
	{
		DIslands cur;
		cudaMemcpy( &cur, W->islDev, sizeof( DIslands ), cudaMemcpyDeviceToHost );
		h = cur;
	}
	size_t ob = h.bodyCap, oc = h.contactCap, oj = h.jointCap;
	size_t nb = d.bodyCap, nc = d.contactCap, nj = d.jointCap;
	if ( ob != nb )
	{
		dgrow( h.bSet, ob, nb );
		dgrow( h.bLocal, ob, nb );
		dgrow( h.bIsland, ob, nb );
		dgrow( h.bIslandPrev, ob, nb );
		dgrow( h.bIslandNext, ob, nb );
		dgrow( h.bHeadContact, ob, nb );
		dgrow( h.bSetNext, ob, nb );
		dgrow( h.bMark, ob, nb );
		dgrow( h.bMoveIndex, ob, nb );
		dgrow( h.islands, ob, nb );
		dgrow( h.islandFree, ob, nb );
		dgrow( h.sets, ob + ( ob ? 8 : 0 ), nb + 8 );
		dgrow( h.setFree, ob + ( ob ? 8 : 0 ), nb + 8 );
		dgrow( h.awakeBodies, ob, nb );
		dgrow( h.awakeIslands, ob, nb );
		dgrow( h.islandBits, 0, nb );
		dgrow( h.stack, 0, nb );
		dgrow( h.seeds, 0, nb );
		dgrow( h.flag, 0, nb );
		dgrow( h.pos, 0, nb );
		dgrow( h.list, 0, nb );
		dgrow( h.moveBody, ob, nb );
		dgrow( h.moveAsleep, ob, nb );
		h.bodyCap = (int)nb;
		h.islandCap = (int)nb;
		h.setCap = (int)nb + 8;
	}
	if ( oc != nc )
	{
		dgrow( h.cSet, oc, nc );
		dgrow( h.cIsland, oc, nc );
		dgrow( h.cIslandPrev, oc, nc );
		dgrow( h.cIslandNext, oc, nc );
		dgrow( h.cSetNext, oc, nc );
		dgrow( h.cMark, oc, nc );
		dgrow( h.cEdge, oc, nc );
		dgrow( h.order, 0, nc );
		dgrow( h.cRemoved, 0, nc );
		h.contactCap = (int)nc;
	}
	if ( oj != nj )
	{
		dgrow( h.jSet, oj, nj );
		dgrow( h.jIsland, oj, nj );
		dgrow( h.jIslandPrev, oj, nj );
		dgrow( h.jIslandNext, oj, nj );
		dgrow( h.jSetNext, oj, nj );
		dgrow( h.jMark, oj, nj );
		dgrow( h.jOverflowIndex, oj, nj );
		h.jointCap = (int)nj;
	}
	if ( h.ncCap < 2 * d.pairCap )
	{
		dfree( h.ncKeys );
		dfree( h.ncKeysAlt );
		dgrow( h.ncKeys, 0, 2 * (size_t)d.pairCap );
		dgrow( h.ncKeysAlt, 0, 2 * (size_t)d.pairCap );
		h.ncCap = 2 * d.pairCap;
	}
	if ( h.logCap < d.bodyCap + d.jointCap )
	{
		dfree( h.log );
		dgrow( h.log, 0, (size_t)d.bodyCap + d.jointCap );
		h.logCap = d.bodyCap + d.jointCap;
	}
	cudaMemcpy( W->islDev, &h, sizeof( DIslands ), cudaMemcpyHostToDevice );
	d.isl = W->islDev;
	d.islFlag = h.flag;
	d.islPos = h.pos;
	d.islNcKeys = h.ncKeys;
	d.islNcKeysAlt = h.ncKeysAlt;
	W->graphDirty = true;
}

static void isl_free( HostWorld* W )
{
	DIslands& h = W->islHost;
	if ( W->islDev )
	{
		int* pi[] = { h.bSet, h.bLocal, h.bIsland, h.bIslandPrev, h.bIslandNext, h.bHeadContact, h.bSetNext, h.bMark,
					  h.bMoveIndex, h.islandFree, h.setFree, h.awakeBodies, h.awakeIslands, h.stack, h.seeds,
					  h.moveBody, h.moveAsleep, h.flag, h.pos, h.list, h.cSet, h.cIsland, h.cIslandPrev, h.cIslandNext, h.cSetNext,
					  h.cMark, h.order, h.jSet, h.jIsland, h.jIslandPrev, h.jIslandNext, h.jSetNext, h.jMark,
					  h.jOverflowIndex, h.log };
		for ( int* p : pi )
			if ( p )
				cudaFree( p );
		if ( h.islands )
			cudaFree( h.islands );
		if ( h.sets )
			cudaFree( h.sets );
		if ( h.cEdge )
			cudaFree( h.cEdge );
		if ( h.islandBits )
			cudaFree( h.islandBits );
		if ( h.cRemoved )
			cudaFree( h.cRemoved );
		if ( h.ncKeys )
			cudaFree( h.ncKeys );
		if ( h.ncKeysAlt )
			cudaFree( h.ncKeysAlt );
		cudaFree( W->islDev );
	}
	W->islDev = nullptr;
	W->d.isl = nullptr;
	W->d.islFlag = W->d.islPos = nullptr;
	W->d.islNcKeys = W->d.islNcKeysAlt = nullptr;
	memset( &h, 0, sizeof( h ) );
}

static void ensure_capacity( HostWorld* W )
{
	bool changed = false;
	DWorld& d = W->d;
	if ( W->bodyCount > d.bodyCap )
	{
		int c = d.bodyCap;
		while ( c < W->bodyCount )
			c *= 2;
		grow_bodies( W, c );
		changed = true;
	}
	if ( W->shapeCount > d.shapeCap )
	{
		int c = d.shapeCap;
		while ( c < W->shapeCount )
			c *= 2;
		grow_shapes( W, c );
		changed = true;
	}
	if ( W->jointCount > d.jointCap )
	{
		int c = d.jointCap;
		while ( c < W->jointCount )
			c *= 2;
		grow_joints( W, c );
		changed = true;
	}
	if ( changed )
	{
		alloc_scratch( W );
		W->graphDirty = true;
	}
	isl_ensure( W );
}

// ---------------------------------------------------------------------------
// ids
// ---------------------------------------------------------------------------
static HostWorld* world_from_id( int32_t worldId )
{
	int index1 = worldId & 0xffff;
	int gen = ( worldId >> 16 ) & 0xffff;
	if ( index1 < 1 || index1 > MAX_WORLDS )
		return nullptr;
	HostWorld* W = s_worlds[index1 - 1];
	if ( W == nullptr || W->used == false || W->generation != gen )
		return nullptr;
	return W;
}

static HostWorld* world_from_wg( int32_t wg )
{
	int world0 = wg & 0xffff;
	if ( world0 < 0 || world0 >= MAX_WORLDS )
		return nullptr;
	HostWorld* W = s_worlds[world0];
	if ( W == nullptr || W->used == false )
		return nullptr;
	return W;
}

static int body_from( int32_t index1, int32_t wg, HostWorld** out )
{
	HostWorld* W = world_from_wg( wg );
	if ( W == nullptr )
		return -1;
	int id = index1 - 1;
	int gen = ( wg >> 16 ) & 0xffff;
	if ( id < 0 || id >= W->bodyCount || ( W->bflags[id] & BF_USED ) == 0 || W->bgen[id] != gen )
		return -1;
	*out = W;
	return id;
}

static int shape_from( int32_t index1, int32_t wg, HostWorld** out )
{
	HostWorld* W = world_from_wg( wg );
	if ( W == nullptr )
		return -1;
	int id = index1 - 1;
	int gen = ( wg >> 16 ) & 0xffff;
	if ( id < 0 || id >= W->shapeCount || ( W->sflags[id] & SF_USED ) == 0 || W->sgen[id] != gen )
		return -1;
	*out = W;
	return id;
}

static int32_t pack_wg( HostWorld* W, int gen )
{
	return ( W->index & 0xffff ) | ( ( gen & 0xffff ) << 16 );
}

// ---------------------------------------------------------------------------
// device row sync
// ---------------------------------------------------------------------------
template <typename T> static void up( T* dptr, const std::vector<T>& h, int lo, int hi, cudaStream_t st, int stride = 1 )
{
	if ( hi <= lo )
		return;
	cudaMemcpyAsync( dptr + (size_t)lo * stride, h.data() + (size_t)lo * stride, sizeof( T ) * (size_t)( hi - lo ) * stride,
					 cudaMemcpyHostToDevice, st );
}

template <typename T> static void down( std::vector<T>& h, const T* dptr, int lo, int hi, int stride = 1 )
{
	if ( hi <= lo )
		return;
	cudaMemcpy( h.data() + (size_t)lo * stride, dptr + (size_t)lo * stride, sizeof( T ) * (size_t)( hi - lo ) * stride,
				cudaMemcpyDeviceToHost );
}

static void upload_body_rows( HostWorld* W, int lo, int hi )
{
	DWorld& d = W->d;
	cudaStream_t st = W->stream;
	up( d.xf, W->xf, lo, hi, st );
	up( d.vel, W->vel, lo, hi, st );
	up( d.delta, W->delta, lo, hi, st );
	up( d.center, W->center, lo, hi, st );
	up( d.sweep0, W->sweep0, lo, hi, st );
	up( d.localCenter, W->localCenter, lo, hi, st );
	up( d.massv, W->massv, lo, hi, st );
	up( d.damp, W->damp, lo, hi, st );
	up( d.bodyGravity, W->bgrav, lo, hi, st );
	up( d.force, W->force, lo, hi, st );
	up( d.bflags, W->bflags, lo, hi, st );
	up( d.headShape, W->headShape, lo, hi, st );
	up( d.headJoint, W->headJoint, lo, hi, st );
	up( d.jointCountB, W->jointCountB, lo, hi, st );
}

static void upload_shape_rows( HostWorld* W, int lo, int hi )
{
	DWorld& d = W->d;
	cudaStream_t st = W->stream;
	up( d.geom, W->geom, lo, hi, st, GEOM_F4 );
	up( d.aabb, W->aabb, lo, hi, st );
	up( d.fat, W->fat, lo, hi, st );
	up( d.mat, W->mat, lo, hi, st );
	up( d.cat, W->cat, lo, hi, st );
	up( d.mask, W->mask, lo, hi, st );
	up( d.group, W->group, lo, hi, st );
	up( d.shapeBody, W->shapeBody, lo, hi, st );
	up( d.shapeSub, W->ssub, lo, hi, st );
	up( d.sflags, W->sflags, lo, hi, st );
	up( d.proxyKey, W->proxyKey, lo, hi, st );
	up( d.nextShape, W->nextShape, lo, hi, st );
}

static void upload_joint_rows( HostWorld* W, int lo, int hi )
{
	DWorld& d = W->d;
	cudaStream_t st = W->stream;
	up( d.jbody, W->jbody, lo, hi, st );
	up( d.jflags, W->jflags, lo, hi, st );
	up( d.jcolor, W->jcolor, lo, hi, st );
	up( d.jnext, W->jnext, lo, hi, st, 2 );
	up( d.jdef0, W->jdef0, lo, hi, st );
	up( d.jdef1, W->jdef1, lo, hi, st );
	up( d.jdef2, W->jdef2, lo, hi, st );
	up( d.jdef3, W->jdef3, lo, hi, st );
}

// bring one existing body's device-updated fields into the host mirror
// The host mirror of the body rows the device changes. After a step or an
// explosion every row may have changed: the first read refreshes the whole
// mirror with one copy per array and later reads are free. After a
// device-side wake or sleep of single bodies, rows are read back one at a
// time until the next step. Rows created or edited on the host since the
// last upload stay authoritative on the host throughout.
enum
{
	MIRROR_FRESH = 0,
	MIRROR_ROWS_STALE = 1,
	MIRROR_ALL_STALE = 2,
};

static void body_rows_changed( HostWorld* W, bool all )
{
	if ( all )
		W->bodyMirror = MIRROR_ALL_STALE;
	else if ( W->bodyMirror == MIRROR_FRESH )
		W->bodyMirror = MIRROR_ROWS_STALE;
}

static void pull_body_rows( HostWorld* W, int lo, int hi )
{
	DWorld& d = W->d;
	down( W->xf, d.xf, lo, hi );
	down( W->vel, d.vel, lo, hi );
	down( W->delta, d.delta, lo, hi );
	down( W->center, d.center, lo, hi );
	down( W->sweep0, d.sweep0, lo, hi );
	down( W->force, d.force, lo, hi );
	down( W->bflags, d.bflags, lo, hi );
}

static void pull_body( HostWorld* W, int b )
{
	if ( b >= W->bodyUploaded || ( b < (int)W->bodyIsDirty.size() && W->bodyIsDirty[b] ) )
		return;
	if ( W->bodyMirror == MIRROR_FRESH )
		return;
	cudaStreamSynchronize( W->stream );
	if ( W->bodyMirror == MIRROR_ROWS_STALE )
	{
		pull_body_rows( W, b, b + 1 );
		return;
	}
	// whole mirror; host-edited rows are kept
	std::vector<int> keep = W->bodyDirty;
	std::vector<float4> kx, kv, kd, ks, kf;
	std::vector<float2> kc;
	std::vector<int> kb;
	for ( int r : keep )
	{
		kx.push_back( W->xf[r] );
		kv.push_back( W->vel[r] );
		kd.push_back( W->delta[r] );
		ks.push_back( W->sweep0[r] );
		kf.push_back( W->force[r] );
		kc.push_back( W->center[r] );
		kb.push_back( W->bflags[r] );
	}
	pull_body_rows( W, 0, W->bodyUploaded );
	for ( size_t k = 0; k < keep.size(); ++k )
	{
		int r = keep[k];
		W->xf[r] = kx[k];
		W->vel[r] = kv[k];
		W->delta[r] = kd[k];
		W->sweep0[r] = ks[k];
		W->force[r] = kf[k];
		W->center[r] = kc[k];
		W->bflags[r] = kb[k];
	}
	W->bodyMirror = MIRROR_FRESH;
}

static void mark_body( HostWorld* W, int b )
{
	if ( b >= W->bodyUploaded )
		return;
	if ( (int)W->bodyIsDirty.size() <= b )
		W->bodyIsDirty.resize( (size_t)W->bodyCount, 0 );
	if ( W->bodyIsDirty[b] == 0 )
	{
		W->bodyIsDirty[b] = 1;
		W->bodyDirty.push_back( b );
	}
}

static void mark_shape( HostWorld* W, int s )
{
	if ( s < W->shapeUploaded )
		W->shapeDirty.push_back( s );
}

// ---------------------------------------------------------------------------
// the broadphase trees between the host copy and the device
// ---------------------------------------------------------------------------
static void pt_free( DProxyTree& T )
{
	dfree( T.child1 );
	dfree( T.child2 );
	dfree( T.parent );
	dfree( T.height );
	dfree( T.flags );
	dfree( T.shape );
	dfree( T.leaves );
	dfree( T.box );
	dfree( T.cat );
	dfree( T.rank );
	dfree( T.rankShape );
	T.cap = 0;
}

static void rb_free( DRebuild& R )
{
	dfree( R.doomed );
	dfree( R.cnt );
	dfree( R.rlc );
	dfree( R.gIdx );
	dfree( R.gCen );
	dfree( R.freed );
	dfree( R.bl );
	dfree( R.br );
	dfree( R.segA );
	dfree( R.segB );
	dfree( R.segSmall );
	dfree( R.chunkBase );
	dfree( R.chunkStat );
	dfree( R.segBounds );
	dfree( R.segBelow );
	dfree( R.pairBase );
	dfree( R.rfStart );
	R.cap = 0;
}

// rebuild scratch for trees of up to `cap` nodes (segments of more than
// 1024 nodes are at most cap / 1024; chunks of 1024 nodes at most
// cap / 1024 plus one per segment)
static void rb_ensure( HostWorld* W, int cap )
{
	DRebuild& R = W->d.rb;
	if ( cap <= R.cap )
		return;
	rb_free( R );
	size_t n = (size_t)cap;
	dgrow( R.doomed, 0, n );
	dgrow( R.cnt, 0, n );
	dgrow( R.rlc, 0, n );
	dgrow( R.gIdx, 0, n );
	dgrow( R.gCen, 0, n );
	dgrow( R.freed, 0, n );
	dgrow( R.bl, 0, n );
	dgrow( R.br, 0, n );
	R.segCap = cap / 512 + 8;
	R.chunkCap = cap / 512 + R.segCap + 8;
	dgrow( R.segA, 0, (size_t)R.segCap );
	dgrow( R.segB, 0, (size_t)R.segCap );
	dgrow( R.segSmall, 0, n / 2 + 8 );
	dgrow( R.chunkBase, 0, (size_t)R.segCap + 1 );
	dgrow( R.chunkStat, 0, 5 * (size_t)R.chunkCap );
	dgrow( R.segBounds, 0, 8 * (size_t)R.segCap ); // two level parities
	dgrow( R.segBelow, 0, 2 * (size_t)R.segCap );
	dgrow( R.pairBase, 0, (size_t)R.segCap + 1 );
	dgrow( R.rfStart, 0, n / 2 + 8 );
	R.cap = cap;
	W->graphDirty = true;
}

// host copy -> device (after host inserts and removes), then the ranks
static void tree_upload( HostWorld* W, int t )
{
	DWorld& d = W->d;
	HTree& h = W->trees[t];
	DProxyTree& T = d.pt[t];
	if ( h.cap > T.cap )
	{
		pt_free( T );
		size_t n = (size_t)h.cap;
		dgrow( T.child1, 0, n );
		dgrow( T.child2, 0, n );
		dgrow( T.parent, 0, n );
		dgrow( T.height, 0, n );
		dgrow( T.flags, 0, n );
		dgrow( T.shape, 0, n );
		dgrow( T.leaves, 0, n );
		dgrow( T.box, 0, n );
		dgrow( T.cat, 0, n );
		dgrow( T.rank, 0, n );
		dgrow( T.rankShape, 0, n );
		T.cap = h.cap;
		W->graphDirty = true;
	}
	int n = h.cap;
	up( T.child1, h.child1, 0, n, W->stream );
	up( T.child2, h.child2, 0, n, W->stream );
	up( T.parent, h.parent, 0, n, W->stream );
	up( T.height, h.height, 0, n, W->stream );
	up( T.flags, h.flags, 0, n, W->stream );
	up( T.shape, h.shape, 0, n, W->stream );
	up( T.leaves, h.leaves, 0, n, W->stream );
	up( T.box, h.box, 0, n, W->stream );
	up( T.cat, h.cat, 0, n, W->stream );
	W->treeScalars[t] = h.root;
	W->treeScalars[3 + t] = h.proxyCount;
	if ( ( d.ptProxies[t] == 0 ) != ( h.proxyCount == 0 ) )
		W->graphDirty = true; // the step launches a tree's rebuild only when it has proxies
	d.ptProxies[t] = h.proxyCount;
	cudaMemcpyAsync( &d.sc->treeRoot[t], &W->treeScalars[t], sizeof( int ), cudaMemcpyHostToDevice, W->stream );
	cudaMemcpyAsync( &d.sc->treeProxies[t], &W->treeScalars[3 + t], sizeof( int ), cudaMemcpyHostToDevice,
					 W->stream );
	launch_pt_ranks( d, W->stream, t );
	rb_ensure( W, std::max( d.pt[1].cap, d.pt[2].cap ) );
	cudaStreamSynchronize( W->stream );
	W->treeDirty[t] = false;
}

// device -> host copy, before a host edit of a tree the steps have changed
static void tree_pull( HostWorld* W, int t )
{
	if ( !W->treeStale[t] )
		return;
	HTree& h = W->trees[t];
	const DProxyTree& T = W->d.pt[t];
	cudaStreamSynchronize( W->stream );
	int n = h.cap;
	down( h.child1, T.child1, 0, n );
	down( h.child2, T.child2, 0, n );
	down( h.parent, T.parent, 0, n );
	down( h.height, T.height, 0, n );
	down( h.flags, T.flags, 0, n );
	down( h.shape, T.shape, 0, n );
	down( h.leaves, T.leaves, 0, n );
	down( h.box, T.box, 0, n );
	down( h.cat, T.cat, 0, n );
	cudaMemcpy( &h.root, &W->d.sc->treeRoot[t], sizeof( int ), cudaMemcpyDeviceToHost );
	W->treeStale[t] = false;
}

// b2BufferMove (broad_phase.c): a proxy joins the next step's move array once
static void host_move( HostWorld* W, int s )
{
	if ( (int)W->hostMoved.size() <= s )
		W->hostMoved.resize( (size_t)s + 1, 0 );
	if ( W->hostMoved[s] )
		return;
	W->hostMoved[s] = 1;
	W->hostMoves.push_back( s );
}

// the buffered proxies go to the device for the step about to be enqueued
static void upload_host_moves( HostWorld* W )
{
	int n = (int)W->hostMoves.size();
	if ( n == 0 )
		return;
	cudaMemcpyAsync( W->d.hostMoves, W->hostMoves.data(), sizeof( int ) * (size_t)n, cudaMemcpyHostToDevice,
					 W->stream );
	W->hostMoveCount = n;
	cudaMemcpyAsync( &W->d.sc->hostMoveCount, &W->hostMoveCount, sizeof( int ), cudaMemcpyHostToDevice, W->stream );
	cudaStreamSynchronize( W->stream );
	for ( int sh : W->hostMoves )
		W->hostMoved[sh] = 0;
	W->hostMoves.clear();
}

static void flush_uploads( HostWorld* W )
{
	ensure_capacity( W );
	if ( W->bodyUploaded < W->bodyCount )
	{
		upload_body_rows( W, W->bodyUploaded, W->bodyCount );
		W->bodyUploaded = W->bodyCount;
		W->islBodiesUploaded = true;
	}
	for ( int b : W->bodyDirty )
	{
		upload_body_rows( W, b, b + 1 );
		W->bodyIsDirty[b] = 0;
		W->islBodiesUploaded = true;
	}
	W->bodyDirty.clear();
	if ( W->shapeUploaded < W->shapeCount )
	{
		upload_shape_rows( W, W->shapeUploaded, W->shapeCount );
		W->shapeUploaded = W->shapeCount;
		W->forceRebuild = true;
	}
	for ( int s : W->shapeDirty )
		upload_shape_rows( W, s, s + 1 );
	if ( !W->shapeDirty.empty() )
		W->forceRebuild = true;
	W->shapeDirty.clear();
	if ( W->jointUploaded < W->jointCount )
	{
		upload_joint_rows( W, W->jointUploaded, W->jointCount );
		W->jointUploaded = W->jointCount;
	}
	for ( int j : W->jointRows )
		upload_joint_rows( W, j, j + 1 );
	W->jointRows.clear();
	if ( !W->islOn && W->awakeOrderDirty )
	{
		int n = (int)W->awakeOrder.size();
		if ( n > 0 )
			cudaMemcpyAsync( W->d.awakeOrder, W->awakeOrder.data(), sizeof( int ) * (size_t)n, cudaMemcpyHostToDevice,
							 W->stream );
		W->awakeOrderCount = n;
		cudaMemcpyAsync( &W->d.sc->awakeOrderCount, &W->awakeOrderCount, sizeof( int ), cudaMemcpyHostToDevice,
						 W->stream );
		cudaStreamSynchronize( W->stream );
		W->awakeOrderDirty = false;
	}
	for ( int j : W->jointDirty )
	{
		DWorld& d = W->d;
		up( d.jdef0, W->jdef0, j, j + 1, W->stream );
		up( d.jdef1, W->jdef1, j, j + 1, W->stream );
		up( d.jdef2, W->jdef2, j, j + 1, W->stream );
		up( d.jdef3, W->jdef3, j, j + 1, W->stream );
		up( d.jflags, W->jflags, j, j + 1, W->stream );
		W->jointIsDirty[j] = 0;
	}
	W->jointDirty.clear();
	if ( W->sensorsDirty )
	{
		// sensor list and overlap buffers; the overlaps of the last step survive
		DWorld& d = W->d;
		int S = (int)W->sensorShapes.size();
		int cap = std::max( 1 << 14, 128 * S );
		if ( d.sensorShapes )
			dfree( d.sensorShapes );
		cudaMalloc( (void**)&d.sensorShapes, sizeof( int ) * (size_t)S );
		cudaMemcpyAsync( d.sensorShapes, W->sensorShapes.data(), sizeof( int ) * (size_t)S, cudaMemcpyHostToDevice,
						 W->stream );
		if ( cap > d.sensorPairCap )
		{
			size_t o = (size_t)d.sensorPairCap;
			dgrow( d.sensorPrevKeys, o, cap );
			dgrow( d.sensorKeys, 0, cap );
			dgrow( d.sensorKeysAlt, 0, cap );
			dgrow( d.sensorBeginEv, 0, cap );
			dgrow( d.sensorEndEv, 0, cap );
			d.sensorPairCap = cap;
		}
		d.sensorCount = S;
		W->sensorsDirty = false;
		W->graphDirty = true;
	}
	if ( W->staticDirty )
	{
		W->trees[0].visit_order( W->staticShapes );
		if ( !W->staticShapes.empty() )
			cudaMemcpyAsync( W->d.staticShapes, W->staticShapes.data(), sizeof( int ) * W->staticShapes.size(),
							 cudaMemcpyHostToDevice, W->stream );
		W->d.staticCount = (int)W->staticShapes.size();
		W->staticDirty = false;
		W->graphDirty = true;
	}
	if ( W->islOn && W->d.isl )
	{
		if ( W->islBodiesUploaded )
		{
			launch_isl_fix_flags( W->d, W->stream, W->bodyCount );
			body_rows_changed( W, false );
		}
		W->islBodiesUploaded = false;
		if ( !W->islLog.empty() )
		{
			int n = (int)W->islLog.size();
			cudaMemcpyAsync( W->islHost.log, W->islLog.data(), sizeof( int ) * n, cudaMemcpyHostToDevice, W->stream );
			W->islLogCount = n;
			cudaMemcpyAsync( &W->islDev->logCount, &W->islLogCount, sizeof( int ), cudaMemcpyHostToDevice, W->stream );
			cudaStreamSynchronize( W->stream );
			launch_isl_create( W->d, W->stream );
			body_rows_changed( W, false );
			W->islLog.clear();
			W->graphDirty = true;
		}
	}
	if ( !W->pendingJoints.empty() )
	{
		cudaMemcpyAsync( W->d.pendingJointOps, W->pendingJoints.data(), sizeof( int ) * W->pendingJoints.size(),
						 cudaMemcpyHostToDevice, W->stream );
		W->d.pendingJointCount = (int)W->pendingJoints.size();
		launch_joint_ops( W->d, W->stream );
		W->d.pendingJointCount = 0;
		W->pendingJoints.clear();
		W->graphDirty = true;
	}
	for ( int t = 0; t < 3; ++t )
		if ( W->treeDirty[t] )
			tree_upload( W, t );
	// counts are kernel parameters of the captured step: a change re-captures
	if ( W->d.bodyCount != W->bodyCount || W->d.shapeCount != W->shapeCount || W->d.jointCount != W->jointCount )
		W->graphDirty = true;
	W->d.bodyCount = W->bodyCount;
	W->d.shapeCount = W->shapeCount;
	W->d.jointCount = W->jointCount;
}

// ---------------------------------------------------------------------------
// world lifecycle
// ---------------------------------------------------------------------------
extern "C" F2D_API int32_t f2d_create_world( const f2d_world_def* def )
{
	int count = 0;
	if ( cudaGetDeviceCount( &count ) != cudaSuccess || count == 0 )
		return 0;
	int slot = -1;
	for ( int i = 0; i < MAX_WORLDS; ++i )
		if ( s_worlds[i] == nullptr || s_worlds[i]->used == false )
		{
			slot = i;
			break;
		}
	if ( slot < 0 )
		return 0;
	uint16_t gen = s_worlds[slot] ? s_worlds[slot]->generation : 0;
	delete s_worlds[slot];
	HostWorld* W = new HostWorld();
	s_worlds[slot] = W;
	W->used = true;
	W->generation = (uint16_t)( gen + 1 );
	W->index = slot;
	W->gridSolverOnly = getenv( "F2D_NO_CLUSTER_SOLVER" ) != nullptr;
	DWorld& d = W->d;
	memset( &d, 0, sizeof( d ) );
	d.gravity = mk( (float)def->gravityX, (float)def->gravityY );
	d.restitutionThreshold = (float)def->restitutionThreshold;
	d.hitEventThreshold = (float)def->hitEventThreshold;
	d.contactHertz = (float)def->contactHertz;
	d.contactDampingRatio = (float)def->contactDampingRatio;
	d.maxContactPushSpeed = (float)def->maxContactPushSpeed;
	d.maxLinearSpeed = (float)def->maximumLinearSpeed;
	d.jointHertz = 60.0f;
	d.jointDampingRatio = 2.0f;
	d.enableSleep = def->enableSleep != 0;
	d.enableContinuous = def->enableContinuous != 0;
	d.enableWarmStarting = 1;
	cudaStreamCreateWithFlags( &W->stream, cudaStreamNonBlocking );
	cudaStreamCreateWithFlags( &W->stream2, cudaStreamNonBlocking );
	cudaEventCreate( &W->evStart );
	cudaEventCreate( &W->evStop );
	cudaEventCreateWithFlags( &W->evFork, cudaEventDisableTiming );
	cudaEventCreateWithFlags( &W->evJoin, cudaEventDisableTiming );
	W->s.rebuild = W->stream2;
	W->s.rebuildFork = W->evFork;
	W->s.rebuildJoin = W->evJoin;
	W->s.rebuildT0 = W->s.rebuildT1 = nullptr;
	cudaEventCreateWithFlags( &W->s.sideFork, cudaEventDisableTiming );
	for ( int k = 0; k < 4; ++k )
	{
		cudaStreamCreateWithFlags( &W->s.side[k], cudaStreamNonBlocking );
		cudaEventCreateWithFlags( &W->s.sideJoin[k], cudaEventDisableTiming );
	}
	cudaMallocHost( (void**)&W->hostError, sizeof( int ) );
	*W->hostError = 0;
	cudaMalloc( (void**)&d.sc, sizeof( DScalars ) );
	cudaMemset( d.sc, 0, sizeof( DScalars ) );
	grow_bodies( W, 1024 );
	grow_shapes( W, 1024 );
	grow_joints( W, 256 );
	alloc_scratch( W );
	// islands and solver sets are kept in worlds created with sleeping on
	W->islOn = def->enableSleep != 0;
	isl_ensure( W );
	return ( slot + 1 ) | ( (int)W->generation << 16 );
}

static void free_world( HostWorld* W )
{
	cudaStreamSynchronize( W->stream );
	if ( W->graphExec )
		cudaGraphExecDestroy( W->graphExec );
	isl_free( W );
	DWorld& d = W->d;
	void** ptrs = (void**)&d;
	(void)ptrs;
	// free every device array
#define F( p ) dfree( d.p )
	F( xf ); F( vel ); F( delta ); F( center ); F( sweep0 ); F( localCenter ); F( massv ); F( damp ); F( force ); F( bodyGravity ); F( shapeSub );
	F( bflags ); F( headShape ); F( headJoint ); F( jointCountB ); F( colorMask ); F( colorLock );
	F( geom ); F( aabb ); F( fat ); F( mat ); F( cat ); F( mask ); F( group ); F( shapeBody ); F( sflags );
	F( proxyKey ); F( nextShape ); F( cshape ); F( cbody ); F( cflags ); F( ccolor ); F( coverflowIndex ); F( cmat );
	F( cmass ); F( mnorm ); F( csimplex ); F( mpA ); F( mpB ); F( mpI ); F( contactFree ); F( pairHash ); F( mortonKeys );
	F( mortonKeysAlt ); F( leafShape ); F( leafShapeAlt ); F( nodeLeft ); F( nodeRight ); F( nodeParent ); F( nodeBox );
	F( nodeVisit ); F( sortHist ); F( pairKeys ); F( pairKeysAlt ); F( pairVal ); F( pairValAlt ); F( planIds );
	F( planKeys ); F( opContact ); F( opKind ); F( opColor ); F( opDone ); F( opBodies ); F( opScan ); F( slotContact ); F( overflowList );
	F( kIndex ); F( kMass ); F( kNormal ); F( kMisc ); F( kSoft ); F( kAnch1 ); F( kAnch2 ); F( kP1 ); F( kP2 );
	F( kImp ); F( kTot ); F( jbody ); F( jflags ); F( jcolor ); F( jcolorSet ); F( jnext ); F( jdef0 ); F( jdef1 ); F( jdef2 ); F( jdef3 );
	F( jimp ); F( jimp2 ); F( jprep0 ); F( jprep1 ); F( jprep2 ); F( jprep3 ); F( jprepM ); F( jindex ); F( overflowJoints ); F( npBucket ); F( ovfOwner ); F( ovfLevel ); F( ovfOrder );
	F( pendingJointOps ); F( fastBodies ); F( beginEv ); F( beginEvF ); F( endEv ); F( hitEvI ); F( hitEvF ); F( moveEvBody );
	F( moveEvXf ); F( staticShapes ); F( sensorShapes ); F( sensorKeys ); F( sensorKeysAlt ); F( sensorPrevKeys );
	F( sensorBeginEv ); F( sensorEndEv ); F( cbList ); F( cbReject ); F( cbManifold ); F( sc ); F( sortTemp ); F( newPoint ); F( newFeat ); F( samples );
	F( shapeMove ); F( moveShape ); F( hostMoves ); F( newPairId ); F( cstamp ); F( awakeOrder ); F( apiEndEv );
#undef F
	for ( int t = 0; t < 3; ++t )
		pt_free( d.pt[t] );
	rb_free( d.rb );
	dfree( W->s.tmpA );
	dfree( W->s.tmpB );
	dfree( W->s.scanTmp );
	dfree( W->s.scanState );
	if ( W->packedBodies )
		cudaFree( W->packedBodies );
	W->packedBodies = nullptr;
	W->packedCap = 0;
	dfree( W->s.bounds );
	cudaFreeHost( W->hostError );
	cudaEventDestroy( W->evStart );
	cudaEventDestroy( W->evStop );
	cudaEventDestroy( W->evFork );
	cudaEventDestroy( W->evJoin );
	cudaEventDestroy( W->s.sideFork );
	for ( int k = 0; k < 4; ++k )
	{
		cudaEventDestroy( W->s.sideJoin[k] );
		cudaStreamDestroy( W->s.side[k] );
	}
	cudaStreamDestroy( W->stream2 );
	cudaStreamDestroy( W->stream );
}

extern "C" F2D_API void f2d_destroy_world( int32_t worldId )
{
	HostWorld* W = world_from_id( worldId );
	if ( W == nullptr )
		return;
	free_world( W );
	uint16_t gen = W->generation;
	int idx = W->index;
	delete W;
	s_worlds[idx] = new HostWorld();
	s_worlds[idx]->generation = gen;
	s_worlds[idx]->used = false;
}

extern "C" F2D_API int32_t f2d_world_is_valid( int32_t worldId )
{
	return world_from_id( worldId ) != nullptr;
}

extern "C" F2D_API void f2d_world_reserve( int32_t worldId, int32_t bodies, int32_t shapes, int32_t contacts,
										   int32_t joints )
{
	HostWorld* W = world_from_id( worldId );
	if ( W == nullptr )
		return;
	cudaStreamSynchronize( W->stream );
	if ( bodies > W->d.bodyCap )
		grow_bodies( W, bodies );
	if ( shapes > W->d.shapeCap )
		grow_shapes( W, shapes );
	if ( contacts > W->d.contactCap )
		grow_contacts( W, contacts );
	if ( joints > W->d.jointCap )
		grow_joints( W, joints );
	alloc_scratch( W );
	isl_ensure( W );
	W->graphDirty = true;
}

// ---------------------------------------------------------------------------
// bodies
// ---------------------------------------------------------------------------
template <typename T> static void vset( std::vector<T>& v, int i, const T& x )
{
	if ( (int)v.size() <= i )
		v.resize( (size_t)i + 1 );
	v[i] = x;
}

// The reference's creation asserts (body.c:180-187, shape.c:166-170, :379-382,
// math_functions.c:10-59) as refusals: a definition they would stop on
// creates nothing and the call returns 0.
static bool valid_float( double v )
{
	return std::isfinite( (float)v );
}

static bool valid_body_def( const f2d_body_def* d )
{
	float c = (float)d->rotationCos, s = (float)d->rotationSin;
	float qq = s * s + c * c;
	return valid_float( d->positionX ) && valid_float( d->positionY ) && valid_float( c ) && valid_float( s ) &&
		   1.0f - 0.0006f < qq && qq < 1.0f + 0.0006f && valid_float( d->linearVelocityX ) &&
		   valid_float( d->linearVelocityY ) && valid_float( d->angularVelocity ) && valid_float( d->linearDamping ) &&
		   d->linearDamping >= 0.0 && valid_float( d->angularDamping ) && d->angularDamping >= 0.0 &&
		   valid_float( d->sleepThreshold ) && d->sleepThreshold >= 0.0 && valid_float( d->gravityScale ) &&
		   d->type >= 0 && d->type <= 2;
}

static bool valid_material( double friction, double restitution, double rolling, double tangentSpeed )
{
	return valid_float( friction ) && friction >= 0.0 && valid_float( restitution ) && restitution >= 0.0 &&
		   valid_float( rolling ) && rolling >= 0.0 && valid_float( tangentSpeed );
}

extern "C" F2D_API int32_t f2d_create_body( int32_t worldId, const f2d_body_def* def, int32_t* index1,
											int32_t* worldAndGeneration )
{
	if ( index1 )
		*index1 = 0;
	if ( worldAndGeneration )
		*worldAndGeneration = 0;
	HostWorld* W = world_from_id( worldId );
	if ( W == nullptr || def == nullptr || !valid_body_def( def ) )
		return 0;
	int id;
	if ( !W->bodyFree.empty() )
	{
		id = W->bodyFree.back();
		W->bodyFree.pop_back();
		pull_body( W, id );
	}
	else
		id = W->bodyCount++;
	uint16_t gen = (uint16_t)( ( id < (int)W->bgen.size() ? W->bgen[id] : 0 ) + 1 );
	vset( W->bgen, id, gen );
	fv2 p = mk( (float)def->positionX, (float)def->positionY );
	frot q;
	q.c = (float)def->rotationCos;
	q.s = (float)def->rotationSin;
	int type = def->type;
	vset( W->xf, id, make_float4( p.x, p.y, q.c, q.s ) );
	float vx = type == 0 ? 0.0f : (float)def->linearVelocityX;
	float vy = type == 0 ? 0.0f : (float)def->linearVelocityY;
	float av = type == 0 ? 0.0f : (float)def->angularVelocity;
	vset( W->vel, id, make_float4( vx, vy, av, 0.0f ) );
	vset( W->delta, id, make_float4( 0.0f, 0.0f, 1.0f, 0.0f ) );
	vset( W->center, id, make_float2( p.x, p.y ) );
	vset( W->sweep0, id, make_float4( p.x, p.y, q.c, q.s ) );
	vset( W->localCenter, id, make_float2( 0.0f, 0.0f ) );
	vset( W->massv, id, make_float4( 0.0f, 0.0f, F2D_HUGE, 0.0f ) );
	vset( W->bgrav, id, W->d.subCount > 0 ? W->subGravity : make_float2( 0.0f, 0.0f ) );
	vset( W->bsub, id, W->d.subCount > 0 ? W->d.subCount - 1 : 0 );
	vset( W->damp, id,
		  make_float4( (float)def->linearDamping, (float)def->angularDamping, (float)def->gravityScale,
					   (float)def->sleepThreshold ) );
	vset( W->force, id, make_float4( 0.0f, 0.0f, 0.0f, 0.0f ) );
	int flags = BF_USED | ( type << BF_TYPE_SHIFT );
	if ( def->isEnabled )
		flags |= BF_ENABLED;
	if ( def->isBullet )
		flags |= BF_BULLET;
	if ( def->allowFastRotation )
		flags |= BF_FAST_ROT;
	if ( def->fixedRotation )
		flags |= BF_FIXED_ROT;
	if ( def->enableSleep )
		flags |= BF_ENABLE_SLEEP;
	if ( W->islOn )
	{
		// a body created asleep starts its own sleeping set (body.c:225-260)
		if ( !def->isAwake && type != 0 && def->isEnabled )
			flags |= BF_ASLEEP;
		W->islLog.push_back( id );
	}
	vset( W->bflags, id, flags );
	vset( W->headShape, id, F2D_NULL );
	vset( W->headJoint, id, F2D_NULL );
	vset( W->headChain, id, F2D_NULL );
	vset( W->jointCountB, id, 0 );
	vset( W->awakeSlot, id, -1 );
	if ( !W->islOn && type != 0 && def->isEnabled )
	{
		// body.c:225-260: a new non-static body joins the awake set's arrays
		W->awakeSlot[id] = (int)W->awakeOrder.size();
		W->awakeOrder.push_back( id );
		W->awakeOrderDirty = true;
	}
	vset( W->bmass, id, 0.0f );
	vset( W->binertia, id, 0.0f );
	mark_body( W, id );
	if ( index1 )
		*index1 = id + 1;
	if ( worldAndGeneration )
		*worldAndGeneration = pack_wg( W, gen );
	return 1;
}

// body.c:528-632 (b2UpdateBodyMassData) on the host mirror
static void update_mass( HostWorld* W, int b )
{
	int type = body_type( W->bflags[b] );
	float mass = 0.0f, inertia = 0.0f, invMass = 0.0f, invInertia = 0.0f;
	fv2 localCenter = mk( 0.0f, 0.0f );
	float minExtent = F2D_HUGE, maxExtent = 0.0f;
	float4 x4 = W->xf[b];
	fxf xf;
	xf.p = mk( x4.x, x4.y );
	xf.q.c = x4.z;
	xf.q.s = x4.w;
	if ( type != 2 )
	{
		W->center[b] = make_float2( xf.p.x, xf.p.y );
		if ( type == 1 )
		{
			for ( int s = W->headShape[b]; s != F2D_NULL; s = W->nextShape[s] )
			{
				float mn, mx;
				h_shape_extent( W->hgeomv[s], mk( 0.0f, 0.0f ), &mn, &mx );
				minExtent = fmin_s( minExtent, mn );
				maxExtent = fmax_s( maxExtent, mx );
			}
		}
		W->bmass[b] = 0.0f;
		W->binertia[b] = 0.0f;
		W->localCenter[b] = make_float2( 0.0f, 0.0f );
		W->massv[b] = make_float4( 0.0f, 0.0f, minExtent, maxExtent );
		return;
	}
	for ( int s = W->headShape[b]; s != F2D_NULL; s = W->nextShape[s] )
	{
		if ( W->density[s] == 0.0f )
			continue;
		HMass md = h_shape_mass( W->hgeomv[s], W->density[s] );
		mass += md.mass;
		localCenter = vmuladd( localCenter, md.mass, md.center );
		inertia += md.rotationalInertia;
	}
	if ( mass > 0.0f )
	{
		invMass = 1.0f / mass;
		localCenter = vscale( invMass, localCenter );
	}
	if ( inertia > 0.0f && ( W->bflags[b] & BF_FIXED_ROT ) == 0 )
	{
		inertia -= mass * vdot( localCenter, localCenter );
		invInertia = 1.0f / inertia;
	}
	else
	{
		inertia = 0.0f;
		invInertia = 0.0f;
	}
	float2 oc = W->center[b];
	fv2 oldCenter = mk( oc.x, oc.y );
	fv2 c = xpoint( xf, localCenter );
	W->localCenter[b] = make_float2( localCenter.x, localCenter.y );
	W->center[b] = make_float2( c.x, c.y );
	float4 s0 = W->sweep0[b];
	W->sweep0[b] = make_float4( c.x, c.y, s0.z, s0.w );
	float4 v = W->vel[b];
	fv2 deltaLinear = vcrossSV( v.z, vsub( c, oldCenter ) );
	W->vel[b] = make_float4( v.x + deltaLinear.x, v.y + deltaLinear.y, v.z, v.w );
	for ( int s = W->headShape[b]; s != F2D_NULL; s = W->nextShape[s] )
	{
		float mn, mx;
		h_shape_extent( W->hgeomv[s], localCenter, &mn, &mx );
		minExtent = fmin_s( minExtent, mn );
		maxExtent = fmax_s( maxExtent, mx );
	}
	W->bmass[b] = mass;
	W->binertia[b] = inertia;
	W->massv[b] = make_float4( invMass, invInertia, minExtent, maxExtent );
}

static void pack_geom( const HShapeGeom& g, float4* out )
{
	for ( int i = 0; i < GEOM_F4; ++i )
		out[i] = make_float4( 0.0f, 0.0f, 0.0f, 0.0f );
	fv2 centroid = h_shape_centroid( g );
	if ( g.type == ST_POLYGON )
	{
		out[0] = make_float4( g.poly.centroid.x, g.poly.centroid.y, 0.0f, 0.0f );
		out[1] = make_float4( g.poly.radius, bits_to_float( g.poly.count ), centroid.x, centroid.y );
		for ( int i = 0; i < 4; ++i )
		{
			out[2 + i] = make_float4( g.poly.v[2 * i].x, g.poly.v[2 * i].y, g.poly.v[2 * i + 1].x, g.poly.v[2 * i + 1].y );
			out[6 + i] = make_float4( g.poly.n[2 * i].x, g.poly.n[2 * i].y, g.poly.n[2 * i + 1].x, g.poly.n[2 * i + 1].y );
		}
	}
	else
	{
		out[0] = make_float4( g.c1.x, g.c1.y, g.c2.x, g.c2.y );
		out[1] = make_float4( g.radius, bits_to_float( 0 ), centroid.x, centroid.y );
		if ( g.type == ST_CHAIN )
			out[2] = make_float4( g.g1.x, g.g1.y, g.g2.x, g.g2.y );
	}
}

// shape.c:59-180 (b2CreateShapeInternal) + shape.c:36-57 (AABBs)
static int create_shape( HostWorld* W, int b, const f2d_shape_def* def, const HShapeGeom& g, int32_t* index1,
						 int32_t* wg )
{
	if ( index1 )
		*index1 = 0;
	if ( wg )
		*wg = 0;
	if ( def == nullptr || !valid_float( def->density ) || def->density < 0.0 ||
		 !valid_material( def->friction, def->restitution, def->rollingResistance, def->tangentSpeed ) )
		return 0;
	pull_body( W, b );
	int id;
	if ( !W->shapeFree.empty() )
	{
		id = W->shapeFree.back();
		W->shapeFree.pop_back();
	}
	else
		id = W->shapeCount++;
	uint16_t gen = (uint16_t)( ( id < (int)W->sgen.size() ? W->sgen[id] : 0 ) + 1 );
	vset( W->sgen, id, gen );
	vset( W->hgeomv, id, g );
	if ( (int)W->geom.size() < ( id + 1 ) * GEOM_F4 )
		W->geom.resize( (size_t)( id + 1 ) * GEOM_F4 );
	pack_geom( g, W->geom.data() + (size_t)id * GEOM_F4 );
	vset( W->mat, id,
		  make_float4( (float)def->friction, (float)def->restitution, (float)def->rollingResistance,
					   (float)def->tangentSpeed ) );
	vset( W->density, id, (float)def->density );
	vset( W->cat, id, (unsigned long long)def->categoryBits );
	vset( W->mask, id, (unsigned long long)def->maskBits );
	vset( W->group, id, def->groupIndex );
	vset( W->shapeBody, id, b );
	vset( W->ssub, id, W->bsub[b] );
	int flags = SF_USED | ( g.type << SF_TYPE_SHIFT );
	if ( def->isSensor )
		flags |= SF_SENSOR;
	if ( def->enableContactEvents )
		flags |= SF_CONTACT_EVENTS;
	if ( def->enableHitEvents )
		flags |= SF_HIT_EVENTS;
	if ( def->enablePreSolveEvents )
		flags |= SF_PRESOLVE;
	if ( def->enableSensorEvents )
		flags |= SF_SENSOR_EVENTS;
	if ( def->isSensor )
	{
		W->sensorShapes.push_back( id );
		W->sensorsDirty = true;
	}
	int pkey = F2D_NULL;
	fbox aabb, fat;
	aabb.lo = aabb.hi = mk( 0.0f, 0.0f );
	fat = aabb;
	int bflags = W->bflags[b];
	if ( bflags & BF_ENABLED )
	{
		int proxyType = body_type( bflags );
		float4 x4 = W->xf[b];
		fxf xf;
		xf.p = mk( x4.x, x4.y );
		xf.q.c = x4.z;
		xf.q.s = x4.w;
		aabb = box_grow( h_shape_aabb( g, xf ), F2D_SPECULATIVE );
		float margin = proxyType == 0 ? F2D_SPECULATIVE : F2D_AABB_MARGIN;
		fat = box_grow( aabb, margin );
		// shape.c:901-911 b2CreateShapeProxy -> broad_phase.c:91-103: the
		// proxy id is the tree node id; non-static (or forced) proxies join
		// the move buffer
		tree_pull( W, proxyType );
		int proxyId = W->trees[proxyType].create_proxy( box_to4( fat ), (unsigned long long)def->categoryBits, id );
		W->treeDirty[proxyType] = true;
		pkey = ( proxyId << 2 ) | proxyType;
		flags |= SF_PROXY;
		bool force = def->invokeContactCreation != 0 || def->isSensor != 0;
		if ( proxyType != 0 || force )
			host_move( W, id );
		if ( proxyType == 0 )
			W->staticDirty = true;
	}
	vset( W->sflags, id, flags );
	vset( W->proxyKey, id, pkey );
	vset( W->aabb, id, box_to4( aabb ) );
	vset( W->fat, id, box_to4( fat ) );
	vset( W->nextShape, id, W->headShape[b] );
	W->headShape[b] = id;
	if ( def->updateBodyMass )
		update_mass( W, b );
	mark_body( W, b );
	mark_shape( W, id );
	if ( index1 )
		*index1 = id + 1;
	if ( wg )
		*wg = pack_wg( W, gen );
	return 1;
}

extern "C" F2D_API int32_t f2d_create_circle_shape( int32_t bi, int32_t bwg, const f2d_shape_def* def, double cx,
													double cy, double radius, int32_t* index1, int32_t* wg )
{
	HostWorld* W;
	int b = body_from( bi, bwg, &W );
	if ( b < 0 || def == nullptr )
		return 0;
	HShapeGeom g = {};
	g.type = ST_CIRCLE;
	g.c1 = mk( (float)cx, (float)cy );
	g.radius = (float)radius;
	return create_shape( W, b, def, g, index1, wg );
}

extern "C" F2D_API int32_t f2d_create_capsule_shape( int32_t bi, int32_t bwg, const f2d_shape_def* def, double x1,
													 double y1, double x2, double y2, double radius, int32_t* index1,
													 int32_t* wg )
{
	HostWorld* W;
	int b = body_from( bi, bwg, &W );
	if ( b < 0 || def == nullptr )
		return 0;
	HShapeGeom g = {};
	g.type = ST_CAPSULE;
	g.c1 = mk( (float)x1, (float)y1 );
	g.c2 = mk( (float)x2, (float)y2 );
	g.radius = (float)radius;
	return create_shape( W, b, def, g, index1, wg );
}

extern "C" F2D_API int32_t f2d_create_segment_shape( int32_t bi, int32_t bwg, const f2d_shape_def* def, double x1,
													 double y1, double x2, double y2, int32_t* index1, int32_t* wg )
{
	HostWorld* W;
	int b = body_from( bi, bwg, &W );
	if ( b < 0 || def == nullptr )
		return 0;
	HShapeGeom g = {};
	g.type = ST_SEGMENT;
	g.c1 = mk( (float)x1, (float)y1 );
	g.c2 = mk( (float)x2, (float)y2 );
	return create_shape( W, b, def, g, index1, wg );
}

// shape.c:339-486 b2CreateChain: count >= 4 points; a loop makes count
// segments, an open chain count - 3 (its end points are ghosts only).
// Materials are six values each (friction, restitution, rollingResistance,
// tangentSpeed, userMaterialId, customColor), one for every segment or one
// per point, a segment taking its leading point's. The segments get the
// default shape definition without contact or hit events and leave the body
// mass alone.
extern "C" F2D_API int32_t f2d_create_chain( int32_t bi, int32_t bwg, const double* points, int32_t count,
											 const double* materials, int32_t materialCount, int64_t categoryBits,
											 int64_t maskBits, int32_t groupIndex, int32_t isLoop,
											 int32_t enableSensorEvents, int32_t* index1, int32_t* wg )
{
	if ( index1 )
		*index1 = 0;
	if ( wg )
		*wg = 0;
	HostWorld* W;
	int b = body_from( bi, bwg, &W );
	if ( b < 0 || points == nullptr || materials == nullptr || count < 4 || count > ( 1 << 20 ) ||
		 ( materialCount != 1 && materialCount != count ) )
		return 0;
	for ( int i = 0; i < materialCount; ++i )
	{
		const double* m = materials + 6 * i;
		if ( !valid_material( m[0], m[1], m[2], m[3] ) )
			return 0;
	}
	int id;
	if ( !W->chainFree.empty() )
	{
		id = W->chainFree.back();
		W->chainFree.pop_back();
	}
	else
	{
		id = (int)W->chainSegments.size();
		W->chainSegments.emplace_back();
		W->chainGen.push_back( 0 );
	}
	W->chainGen[id] = (uint16_t)( W->chainGen[id] + 1 );
	vset( W->chainBody, id, b );
	vset( W->chainNext, id, W->headChain[b] );
	W->headChain[b] = id;
	std::vector<int>& segs = W->chainSegments[id];
	segs.clear();
	int n = isLoop ? count : count - 3;
	f2d_shape_def d = {};
	d.density = 1.0;
	d.categoryBits = categoryBits;
	d.maskBits = maskBits;
	d.groupIndex = groupIndex;
	d.enableSensorEvents = enableSensorEvents != 0;
	d.invokeContactCreation = 1;
	d.updateBodyMass = 0;
	auto pt = [&]( int i ) { return mk( (float)points[2 * i], (float)points[2 * i + 1] ); };
	for ( int k = 0; k < n; ++k )
	{
		int i0, i1, i2, i3, mi;
		if ( isLoop )
		{
			i0 = ( k + count - 1 ) % count;
			i1 = k;
			i2 = ( k + 1 ) % count;
			i3 = ( k + 2 ) % count;
			mi = k;
		}
		else
		{
			i0 = k;
			i1 = k + 1;
			i2 = k + 2;
			i3 = k + 3;
			mi = k + 1;
		}
		const double* m = materials + 6 * ( materialCount == 1 ? 0 : mi );
		d.friction = m[0];
		d.restitution = m[1];
		d.rollingResistance = m[2];
		d.tangentSpeed = m[3];
		d.userMaterialId = (int)m[4];
		HShapeGeom g = {};
		g.type = ST_CHAIN;
		g.g1 = pt( i0 );
		g.c1 = pt( i1 );
		g.c2 = pt( i2 );
		g.g2 = pt( i3 );
		int32_t si = 0, swg = 0;
		create_shape( W, b, &d, g, &si, &swg );
		segs.push_back( si - 1 );
	}
	if ( index1 )
		*index1 = id + 1;
	if ( wg )
		*wg = pack_wg( W, W->chainGen[id] );
	return 1;
}

// RawBox2D.chainGetSegments (raw_box2d.dart:571): segment shape ids as
// (index1, worldAndGeneration) pairs; returns the segment count
extern "C" F2D_API int32_t f2d_chain_get_segments( int32_t index1, int32_t wg, int32_t* out2, int32_t capacity )
{
	HostWorld* W = world_from_wg( wg );
	if ( W == nullptr )
		return 0;
	int id = index1 - 1;
	if ( id < 0 || id >= (int)W->chainSegments.size() || W->chainGen[id] != ( ( wg >> 16 ) & 0xffff ) )
		return 0;
	const std::vector<int>& segs = W->chainSegments[id];
	int n = (int)segs.size();
	for ( int i = 0; i < n && i < capacity && out2 != nullptr; ++i )
	{
		out2[2 * i] = segs[i] + 1;
		out2[2 * i + 1] = pack_wg( W, W->sgen[segs[i]] );
	}
	return n;
}

extern "C" F2D_API int32_t f2d_create_box_shape( int32_t bi, int32_t bwg, const f2d_shape_def* def, double hx,
												 double hy, double cx, double cy, double c, double s, double radius,
												 int32_t* index1, int32_t* wg )
{
	HostWorld* W;
	int b = body_from( bi, bwg, &W );
	if ( b < 0 || def == nullptr || !valid_float( radius ) || radius < 0.0 ) // shape.c:213
		return 0;
	HShapeGeom g = {};
	g.type = ST_POLYGON;
	frot q;
	q.c = (float)c;
	q.s = (float)s;
	g.poly = h_make_offset_rounded_box( (float)hx, (float)hy, mk( (float)cx, (float)cy ), q, (float)radius );
	return create_shape( W, b, def, g, index1, wg );
}

extern "C" F2D_API int32_t f2d_create_polygon_shape( int32_t bi, int32_t bwg, const f2d_shape_def* def,
													 const double* points, int32_t count, double radius,
													 int32_t* index1, int32_t* wg )
{
	if ( index1 )
		*index1 = 0;
	if ( wg )
		*wg = 0;
	HostWorld* W;
	int b = body_from( bi, bwg, &W );
	if ( b < 0 || def == nullptr || points == nullptr || count < 3 || count > F2D_MAX_POLY || !valid_float( radius ) ||
		 radius < 0.0 ) // shape.c:213
		return 0;
	fv2 pts[F2D_MAX_POLY], hull[F2D_MAX_POLY];
	for ( int i = 0; i < count; ++i )
		pts[i] = mk( (float)points[2 * i], (float)points[2 * i + 1] );
	int hc = h_compute_hull( pts, count, hull );
	if ( hc == 0 )
		return 0;
	HShapeGeom g = {};
	g.type = ST_POLYGON;
	g.poly = h_make_polygon( hull, hc, (float)radius );
	return create_shape( W, b, def, g, index1, wg );
}

extern "C" F2D_API int32_t f2d_shape_is_valid( int32_t index1, int32_t wg )
{
	HostWorld* W;
	return shape_from( index1, wg, &W ) >= 0;
}

extern "C" F2D_API int32_t f2d_shape_get_type( int32_t index1, int32_t wg )
{
	HostWorld* W;
	int s = shape_from( index1, wg, &W );
	if ( s < 0 )
		return -1;
	return shape_type( W->sflags[s] );
}

// ---------------------------------------------------------------------------
// joints (joint.c:146-330, :507-560)
// ---------------------------------------------------------------------------
// Shared tail of the joint constructors (joint.c:146-330): slot, generation,
// body joint lists, definition rows, then the graph / island log.
static void destroy_contacts_between( HostWorld* W, int a, int b );

static int create_joint_common( HostWorld* W, int a, int b, int flags, float4 d0, float4 d1, float4 d2,
								int32_t* index1, int32_t* wg, float4 d3 = make_float4( 0.0f, 0.0f, 0.0f, 0.0f ) )
{
	int j;
	if ( !W->jointFree.empty() )
	{
		j = W->jointFree.back();
		W->jointFree.pop_back();
		if ( j < W->jointUploaded )
			W->jointRows.push_back( j );
	}
	else
		j = W->jointCount++;
	uint16_t gen = (uint16_t)( ( j < (int)W->jgen.size() ? W->jgen[j] : 0 ) + 1 );
	vset( W->jgen, j, gen );
	vset( W->jbody, j, make_int2( a, b ) );
	vset( W->jflags, j, flags );
	vset( W->jcolor, j, F2D_NULL );
	if ( (int)W->jnext.size() < 2 * ( j + 1 ) )
		W->jnext.resize( 2 * ( (size_t)j + 1 ) );
	pull_body( W, a );
	pull_body( W, b );
	W->jnext[2 * j + 0] = W->headJoint[a];
	W->headJoint[a] = ( j << 1 ) | 0;
	W->jointCountB[a] += 1;
	W->jnext[2 * j + 1] = W->headJoint[b];
	W->headJoint[b] = ( j << 1 ) | 1;
	W->jointCountB[b] += 1;
	mark_body( W, a );
	mark_body( W, b );
	vset( W->jdef0, j, d0 );
	vset( W->jdef1, j, d1 );
	vset( W->jdef2, j, d2 );
	vset( W->jdef3, j, d3 );
	// joints between two static bodies or with a disabled body never enter
	// the graph
	bool staticA = body_type( W->bflags[a] ) == 0, staticB = body_type( W->bflags[b] ) == 0;
	bool enabled = ( W->bflags[a] & BF_ENABLED ) && ( W->bflags[b] & BF_ENABLED );
	if ( W->islOn )
		W->islLog.push_back( ( 1 << 30 ) | j ); // set, colour and island at the next upload
	else if ( !( staticA && staticB ) && enabled )
		W->pendingJoints.push_back( j );
	// joint.c:396-400 and the other constructors but the mouse and filter
	// joints: contacts between bodies that may no longer collide go
	int type = ( flags >> JF_TYPE_SHIFT ) & 0xf;
	if ( ( flags & JF_COLLIDE ) == 0 && type != F2D_JOINT_MOUSE && type != F2D_JOINT_FILTER )
		destroy_contacts_between( W, a, b );
	if ( index1 )
		*index1 = j + 1;
	if ( wg )
		*wg = pack_wg( W, gen );
	return 1;
}

static HostWorld* joint_bodies( int32_t worldId, int32_t aIndex1, int32_t aWg, int32_t bIndex1, int32_t bWg, int* a,
								int* b )
{
	HostWorld* W = world_from_id( worldId );
	if ( W == nullptr )
		return nullptr;
	HostWorld* WA;
	HostWorld* WB;
	*a = body_from( aIndex1, aWg, &WA );
	*b = body_from( bIndex1, bWg, &WB );
	if ( *a < 0 || *b < 0 || WA != W || WB != W )
		return nullptr;
	return W;
}

extern "C" F2D_API int32_t f2d_create_revolute_joint( int32_t worldId, const f2d_revolute_def* def, int32_t* index1,
													  int32_t* wg )
{
	if ( index1 )
		*index1 = 0;
	if ( wg )
		*wg = 0;
	if ( def == nullptr )
		return 0;
	int a, b;
	HostWorld* W = joint_bodies( worldId, def->bodyAIndex1, def->bodyAWorldAndGeneration, def->bodyBIndex1,
								 def->bodyBWorldAndGeneration, &a, &b );
	if ( W == nullptr )
		return 0;
	int flags = JF_USED;
	if ( def->enableSpring )
		flags |= JF_SPRING;
	if ( def->enableLimit )
		flags |= JF_LIMIT;
	if ( def->enableMotor )
		flags |= JF_MOTOR;
	if ( def->collideConnected )
		flags |= JF_COLLIDE;
	float ref = fclamp_s( (float)def->referenceAngle, -F2D_PI, F2D_PI );
	float target = fclamp_s( (float)def->targetAngle, -F2D_PI, F2D_PI );
	return create_joint_common(
		W, a, b, flags,
		make_float4( (float)def->localAnchorAX, (float)def->localAnchorAY, (float)def->localAnchorBX,
					 (float)def->localAnchorBY ),
		make_float4( ref, target, (float)def->hertz, (float)def->dampingRatio ),
		make_float4( (float)def->lowerAngle, (float)def->upperAngle, (float)def->maxMotorTorque, (float)def->motorSpeed ),
		index1, wg );
}

// b2Create{Weld,Distance,Prismatic,Wheel,Motor,Mouse,Filter}Joint
// (joint.c:400-720): distance lengths clamped to the linear slop with
// maxLength at least minLength; joint axes normalised; the motor joint's
// anchors at the body origins and its correction factor clamped to [0, 1];
// the mouse joint's anchors are the target in each body's frame at creation;
// the filter joint never lets its bodies collide. Definition rows per type:
//   weld       d1 referenceAngle linearHertz linearDampingRatio angularHertz
//              d2 angularDampingRatio
//   distance   d1 length minLength maxLength hertz
//              d2 dampingRatio maxMotorForce motorSpeed
//   prismatic  d1 localAxisA.xy referenceAngle targetTranslation
//              d2 lowerTranslation upperTranslation maxMotorForce motorSpeed
//              d3 hertz dampingRatio
//   wheel      d1 localAxisA.xy hertz dampingRatio
//              d2 lowerTranslation upperTranslation maxMotorTorque motorSpeed
//   motor      d1 linearOffset.xy angularOffset maxForce
//              d2 maxTorque correctionFactor
//   mouse      d1 target.xy hertz dampingRatio
//              d2 maxForce
extern "C" F2D_API int32_t f2d_create_joint( int32_t worldId, const f2d_joint_def* def, int32_t* index1, int32_t* wg )
{
	if ( index1 )
		*index1 = 0;
	if ( wg )
		*wg = 0;
	if ( def == nullptr || def->type < F2D_JOINT_WELD || def->type > F2D_JOINT_FILTER )
		return 0;
	int a, b;
	HostWorld* W = joint_bodies( worldId, def->bodyAIndex1, def->bodyAWorldAndGeneration, def->bodyBIndex1,
								 def->bodyBWorldAndGeneration, &a, &b );
	if ( W == nullptr )
		return 0;
	int type = def->type;
	int flags = JF_USED | ( type << JF_TYPE_SHIFT );
	if ( def->collideConnected && type != F2D_JOINT_FILTER )
		flags |= JF_COLLIDE;
	if ( type == F2D_JOINT_DISTANCE || type == F2D_JOINT_PRISMATIC || type == F2D_JOINT_WHEEL )
	{
		if ( def->enableSpring )
			flags |= JF_SPRING;
		if ( def->enableLimit )
			flags |= JF_LIMIT;
		if ( def->enableMotor )
			flags |= JF_MOTOR;
	}
	const float4 zero = make_float4( 0.0f, 0.0f, 0.0f, 0.0f );
	float4 d0 = make_float4( (float)def->localAnchorAX, (float)def->localAnchorAY, (float)def->localAnchorBX,
							 (float)def->localAnchorBY );
	float4 d1 = zero, d2 = zero, d3 = zero;
	fv2 axis = vnormalize( mk( (float)def->localAxisAX, (float)def->localAxisAY ) );
	switch ( type )
	{
		case F2D_JOINT_WELD:
			d1 = make_float4( (float)def->referenceAngle, (float)def->linearHertz, (float)def->linearDampingRatio,
							  (float)def->angularHertz );
			d2 = make_float4( (float)def->angularDampingRatio, 0.0f, 0.0f, 0.0f );
			break;
		case F2D_JOINT_DISTANCE:
			d1 = make_float4( fmax_s( (float)def->length, F2D_LINEAR_SLOP ),
							  fmax_s( (float)def->minLength, F2D_LINEAR_SLOP ),
							  fmax_s( (float)def->minLength, (float)def->maxLength ), (float)def->hertz );
			d2 = make_float4( (float)def->dampingRatio, (float)def->maxMotorForce, (float)def->motorSpeed, 0.0f );
			break;
		case F2D_JOINT_PRISMATIC:
			d1 = make_float4( axis.x, axis.y, (float)def->referenceAngle, (float)def->targetTranslation );
			d2 = make_float4( (float)def->lowerTranslation, (float)def->upperTranslation, (float)def->maxMotorForce,
							  (float)def->motorSpeed );
			d3 = make_float4( (float)def->hertz, (float)def->dampingRatio, 0.0f, 0.0f );
			break;
		case F2D_JOINT_WHEEL:
			d1 = make_float4( axis.x, axis.y, (float)def->hertz, (float)def->dampingRatio );
			d2 = make_float4( (float)def->lowerTranslation, (float)def->upperTranslation, (float)def->maxMotorTorque,
							  (float)def->motorSpeed );
			break;
		case F2D_JOINT_MOTOR:
			d0 = zero;
			d1 = make_float4( (float)def->linearOffsetX, (float)def->linearOffsetY, (float)def->angularOffset,
							  (float)def->maxForce );
			d2 = make_float4( (float)def->maxTorque, fclamp_s( (float)def->correctionFactor, 0.0f, 1.0f ), 0.0f, 0.0f );
			break;
		case F2D_JOINT_MOUSE:
		{
			pull_body( W, a );
			pull_body( W, b );
			float tx = (float)def->targetX, ty = (float)def->targetY;
			float4 xa = W->xf[a], xb = W->xf[b];
			float ax = tx - xa.x, ay = ty - xa.y;
			float bx = tx - xb.x, by = ty - xb.y;
			d0 = make_float4( xa.z * ax + xa.w * ay, -xa.w * ax + xa.z * ay, xb.z * bx + xb.w * by,
							  -xb.w * bx + xb.z * by );
			d1 = make_float4( tx, ty, (float)def->hertz, (float)def->dampingRatio );
			d2 = make_float4( (float)def->maxForce, 0.0f, 0.0f, 0.0f );
			break;
		}
		default: // filter
			d0 = zero;
			break;
	}
	return create_joint_common( W, a, b, flags, d0, d1, d2, index1, wg, d3 );
}

// a live joint of generation wg (j below the joint count)
static bool joint_live( const HostWorld* W, int j, int32_t wg )
{
	return ( W->jflags[j] & JF_USED ) != 0 && W->jgen[j] == ( ( wg >> 16 ) & 0xffff );
}

// an uploaded joint whose definition rows changed on the host (sent with the
// next step)
static void mark_joint_dirty( HostWorld* W, int j )
{
	if ( j >= W->jointUploaded )
		return;
	if ( (int)W->jointIsDirty.size() <= j )
		W->jointIsDirty.resize( (size_t)j + 1, 0 );
	if ( W->jointIsDirty[j] )
		return;
	W->jointIsDirty[j] = 1;
	W->jointDirty.push_back( j );
}

// Limit of a revolute, prismatic or wheel joint (revolute_joint.c:84-127,
// prismatic_joint.c:68-109, wheel_joint.c:57-98): EnableLimit then SetLimits;
// a change clears the limit impulses (jimp2); bounds stored as min, max.
extern "C" F2D_API void f2d_joint_set_limits( int32_t index1, int32_t wg, int32_t enable, double lower, double upper )
{
	HostWorld* W = world_from_wg( wg );
	if ( W == nullptr )
		return;
	int j = index1 - 1;
	if ( j < 0 || j >= W->jointCount || !joint_live( W, j, wg ) )
		return;
	int type = ( W->jflags[j] >> JF_TYPE_SHIFT ) & 0xf;
	if ( type != 0 && type != F2D_JOINT_PRISMATIC && type != F2D_JOINT_WHEEL )
		return;
	bool clear = false;
	if ( ( enable != 0 ) != ( ( W->jflags[j] & JF_LIMIT ) != 0 ) )
	{
		W->jflags[j] ^= JF_LIMIT;
		clear = true;
	}
	float lo = (float)lower, hi = (float)upper;
	float4& d2 = W->jdef2[j];
	if ( lo != d2.x || hi != d2.y )
	{
		d2.x = fmin_s( lo, hi );
		d2.y = fmax_s( lo, hi );
		clear = true;
	}
	// stream-ordered clear: after any step in flight, before the next one,
	// without blocking the caller
	if ( clear && j < W->jointUploaded )
		cudaMemsetAsync( W->d.jimp2 + j, 0, sizeof( float2 ), W->stream );
	mark_joint_dirty( W, j );
}

// b2Joint_GetConstraintForce / GetConstraintTorque (joint.c:1061-1135) with
// the per-type b2Get*JointForce / Torque: the last step's impulses times its
// inverse substep; out3 = force.x, force.y, torque
extern "C" F2D_API void f2d_joint_get_constraint( int32_t index1, int32_t wg, float* out3 )
{
	out3[0] = out3[1] = out3[2] = 0.0f;
	HostWorld* W = world_from_wg( wg );
	if ( W == nullptr )
		return;
	int j = index1 - 1;
	if ( j < 0 || j >= W->jointCount || !joint_live( W, j, wg ) || j >= W->jointUploaded )
		return;
	cudaStreamSynchronize( W->stream );
	float4 imp, p3;
	float2 imp2;
	cudaMemcpy( &imp, W->d.jimp + j, sizeof( imp ), cudaMemcpyDeviceToHost );
	cudaMemcpy( &imp2, W->d.jimp2 + j, sizeof( imp2 ), cudaMemcpyDeviceToHost );
	cudaMemcpy( &p3, W->d.jprep3 + j, sizeof( p3 ), cudaMemcpyDeviceToHost );
	int type = ( W->jflags[j] >> JF_TYPE_SHIFT ) & 0xf;
	int a = W->jbody[j].x, b = W->jbody[j].y;
	float inv_h = W->invH;
	fv2 f = mk( 0.0f, 0.0f );
	float t = 0.0f;
	auto xf_of = [&]( int body ) {
		pull_body( W, body );
		float4 x = W->xf[body];
		fxf r;
		r.p = mk( x.x, x.y );
		r.q.c = x.z;
		r.q.s = x.w;
		return r;
	};
	switch ( type )
	{
		case 0: // revolute_joint.c:176-187
			f = vscale( inv_h, mk( imp.x, imp.y ) );
			t = inv_h * ( imp.w + imp2.x - imp2.y );
			break;
		case F2D_JOINT_WELD:  // weld_joint.c:66-75
		case F2D_JOINT_MOTOR: // motor_joint.c:74-83
		case F2D_JOINT_MOUSE: // mouse_joint.c:66-75
			f = vscale( inv_h, mk( imp.x, imp.y ) );
			t = inv_h * imp.z;
			break;
		case F2D_JOINT_DISTANCE: // distance_joint.c:185-198
		{
			float4 d0 = W->jdef0[j];
			fv2 pA = xpoint( xf_of( a ), mk( d0.x, d0.y ) );
			fv2 pB = xpoint( xf_of( b ), mk( d0.z, d0.w ) );
			fv2 axis = vnormalize( vsub( pB, pA ) );
			float force = ( imp.x + imp.y - imp.z + imp.w ) * inv_h;
			f = vscale( force, axis );
			break;
		}
		case F2D_JOINT_PRISMATIC: // prismatic_joint.c:211-232
		{
			float4 d1 = W->jdef1[j];
			fv2 axisA = rrot( xf_of( a ).q, mk( d1.x, d1.y ) );
			fv2 perpA = vleft( axisA );
			float perpForce = inv_h * imp.x;
			float axialForce = inv_h * ( imp.w + imp2.x - imp2.y );
			f = vadd( vscale( perpForce, perpA ), vscale( axialForce, axisA ) );
			t = inv_h * imp.y;
			break;
		}
		case F2D_JOINT_WHEEL: // wheel_joint.c:147-165 (axis of the last step)
		{
			fv2 axisA = mk( p3.x, p3.y );
			fv2 perpA = vleft( axisA );
			float perpForce = inv_h * imp.x;
			float axialForce = inv_h * ( imp.y + imp2.x - imp2.y );
			f = vadd( vscale( perpForce, perpA ), vscale( axialForce, axisA ) );
			t = inv_h * imp.z;
			break;
		}
		default:
			break;
	}
	out3[0] = f.x;
	out3[1] = f.y;
	out3[2] = t;
}

// Motor of a revolute, prismatic, wheel or distance joint (revolute_joint.c:
// 129-168, prismatic_joint.c:111-150, wheel_joint.c:100-140, distance_joint.c:
// 138-175): speed and the maximum torque (revolute, wheel) or force
// (prismatic, distance); switching the motor clears its impulse. No wake.
extern "C" F2D_API void f2d_joint_set_motor( int32_t index1, int32_t wg, int32_t enable, double speed, double maxMotor )
{
	HostWorld* W = world_from_wg( wg );
	if ( W == nullptr )
		return;
	int j = index1 - 1;
	if ( j < 0 || j >= W->jointCount || !joint_live( W, j, wg ) )
		return;
	int type = ( W->jflags[j] >> JF_TYPE_SHIFT ) & 0xf;
	float4& d2 = W->jdef2[j];
	int impulseLane; // the motor impulse's component of the jimp row
	if ( type == 0 || type == F2D_JOINT_PRISMATIC || type == F2D_JOINT_WHEEL )
	{
		d2.z = (float)maxMotor;
		d2.w = (float)speed;
		impulseLane = type == F2D_JOINT_WHEEL ? 2 : 3;
	}
	else if ( type == F2D_JOINT_DISTANCE )
	{
		d2.y = (float)maxMotor;
		d2.z = (float)speed;
		impulseLane = 3;
	}
	else
		return;
	bool on = ( W->jflags[j] & JF_MOTOR ) != 0;
	if ( ( enable != 0 ) != on )
	{
		W->jflags[j] ^= JF_MOTOR;
		// stream-ordered clear, as in f2d_joint_set_limits
		if ( j < W->jointUploaded )
			cudaMemsetAsync( (float*)( W->d.jimp + j ) + impulseLane, 0, sizeof( float ), W->stream );
	}
	mark_joint_dirty( W, j );
}

// b2MouseJoint_SetTarget (mouse_joint.c:14-19): no wake
extern "C" F2D_API void f2d_mouse_joint_set_target( int32_t index1, int32_t wg, double x, double y )
{
	HostWorld* W = world_from_wg( wg );
	if ( W == nullptr )
		return;
	int j = index1 - 1;
	if ( j < 0 || j >= W->jointCount || !joint_live( W, j, wg ) ||
		 ( ( W->jflags[j] >> JF_TYPE_SHIFT ) & 0xf ) != F2D_JOINT_MOUSE )
		return;
	W->jdef1[j].x = (float)x;
	W->jdef1[j].y = (float)y;
	mark_joint_dirty( W, j );
}

extern "C" F2D_API int32_t f2d_joint_is_valid( int32_t index1, int32_t wg )
{
	HostWorld* W = world_from_wg( wg );
	if ( W == nullptr )
		return 0;
	int j = index1 - 1;
	return j >= 0 && j < W->jointCount && ( W->jflags[j] & JF_USED ) && W->jgen[j] == ( ( wg >> 16 ) & 0xffff );
}

// ---------------------------------------------------------------------------
// destroy path: b2DestroyBody (body.c:343-440), b2DestroyShape and
// b2DestroyShapeInternal (shape.c:230-338), b2DestroyChain (:488-540),
// b2DestroyJoint and b2DestroyJointInternal (joint.c:702-822),
// b2DestroyContactsBetweenBodies (:313-351), b2DestroySensor
// (sensor.c:353-380), b2BroadPhase_DestroyProxy (broad_phase.c:70-114).
// The host keeps the id pools, the body shape, joint and chain lists, the
// trees and the sensor list; the device takes contacts, joints and bodies out
// of the constraint graph, the islands and the solver sets in the
// reference's order (island.cu). Single fields go up as they change, so
// device-side state (positions, sleep timers) is never overwritten.
// ---------------------------------------------------------------------------
static bool chain_live( const HostWorld* W, int c, int32_t wg )
{
	return c >= 0 && c < (int)W->chainSegments.size() && W->chainBody[c] >= 0 &&
		   W->chainGen[c] == ( ( wg >> 16 ) & 0xffff );
}

// creations reach the device and the proxies buffered since the last step
// join the move array (after the finalize moves, as b2BufferMove appends)
static void destroy_begin( HostWorld* W )
{
	flush_uploads( W );
	if ( !W->hostMoves.empty() )
	{
		upload_host_moves( W );
		launch_pt_host_moves( W->d, W->s, W->stream );
	}
	cudaMemsetAsync( &W->d.sc->apiEndCount, 0, sizeof( int ), W->stream );
	cudaMemsetAsync( &W->d.sc->apiCount, 0, sizeof( int ), W->stream );
}

// end events of the contacts destroyed since destroy_begin, with the shape
// ids as they are now, for the next step's events
static void destroy_end( HostWorld* W )
{
	cudaStreamSynchronize( W->stream );
	int n = 0;
	cudaMemcpy( &n, &W->d.sc->apiEndCount, sizeof( int ), cudaMemcpyDeviceToHost );
	n = std::min( n, W->d.contactCap );
	if ( n > 0 )
	{
		std::vector<int> ev( 2 * (size_t)n );
		cudaMemcpy( ev.data(), W->d.apiEndEv, sizeof( int ) * 2 * (size_t)n, cudaMemcpyDeviceToHost );
		for ( int i = 0; i < n; ++i )
		{
			int a = ev[2 * i], b = ev[2 * i + 1];
			W->endNext.insert( W->endNext.end(),
							   { a + 1, pack_wg( W, W->sgen[a] ), b + 1, pack_wg( W, W->sgen[b] ) } );
		}
	}
	if ( W->islOn )
		body_rows_changed( W, false ); // woken sets
	W->forceRebuild = true;
}

// the joint key leaves body b's joint list (singly linked here)
static void unlink_joint_key( HostWorld* W, int b, int key, int next )
{
	if ( W->headJoint[b] == key )
	{
		W->headJoint[b] = next;
		up( W->d.headJoint, W->headJoint, b, b + 1, W->stream );
		return;
	}
	for ( int cur = W->headJoint[b], g = 0; cur != F2D_NULL && g <= W->jointCount; ++g )
	{
		int slot = 2 * ( cur >> 1 ) + ( cur & 1 );
		if ( W->jnext[slot] == key )
		{
			W->jnext[slot] = next;
			up( W->d.jnext, W->jnext, slot, slot + 1, W->stream );
			return;
		}
		cur = W->jnext[slot];
	}
}

static void destroy_joint_host( HostWorld* W, int j, int wake )
{
	int2 jb = W->jbody[j];
	int ids[2] = { jb.x, jb.y };
	for ( int e = 0; e < 2; ++e )
	{
		int b = ids[e];
		unlink_joint_key( W, b, ( j << 1 ) | e, W->jnext[2 * j + e] );
		W->jointCountB[b] -= 1;
		up( W->d.jointCountB, W->jointCountB, b, b + 1, W->stream );
	}
	launch_destroy_joint( W->d, W->stream, j, wake );
	W->jflags[j] = 0;
	W->jcolor[j] = F2D_NULL;
	W->jointFree.push_back( j );
}

// broad_phase.c:105-114: out of the move array, then out of its tree
static void destroy_proxy_host( HostWorld* W, int s )
{
	int pk = W->proxyKey[s];
	if ( pk == F2D_NULL )
		return;
	launch_unbuffer_move( W->d, W->stream, s );
	int t = pk & 3;
	tree_pull( W, t );
	W->trees[t].destroy_proxy( pk >> 2 );
	W->treeDirty[t] = true;
	if ( t == 0 )
		W->staticDirty = true;
	W->proxyKey[s] = F2D_NULL;
	up( W->d.proxyKey, W->proxyKey, s, s + 1, W->stream );
}

// sensor.c:353-380: an end event per current visitor (the last step's
// overlaps, visitor order), then the sensor leaves the sensor array by
// swap-remove and the overlaps of the moved sensor follow it
static void destroy_sensor_host( HostWorld* W, int s )
{
	std::vector<int>& S = W->sensorShapes;
	int idx = -1;
	for ( int i = 0; i < (int)S.size(); ++i )
		if ( S[i] == s )
			idx = i;
	if ( idx < 0 )
		return;
	int last = (int)S.size() - 1;
	DWorld& d = W->d;
	if ( W->stepped && d.sensorCount > 0 && d.sensorPrevKeys )
	{
		cudaStreamSynchronize( W->stream );
		int n = 0;
		cudaMemcpy( &n, &d.sc->sensorPrev, sizeof( int ), cudaMemcpyDeviceToHost );
		n = std::max( 0, std::min( n, d.sensorPairCap ) );
		std::vector<unsigned long long> keys( (size_t)n ), kept;
		if ( n > 0 )
			cudaMemcpy( keys.data(), d.sensorPrevKeys, sizeof( unsigned long long ) * (size_t)n, cudaMemcpyDeviceToHost );
		for ( unsigned long long k : keys )
		{
			int si = (int)( k >> 32 );
			int v = (int)( k & 0xffffffffull );
			if ( si == idx )
			{
				W->sensorEndNext.insert( W->sensorEndNext.end(),
										 { s + 1, pack_wg( W, W->sgen[s] ), v + 1, pack_wg( W, W->sgen[v] ) } );
				continue;
			}
			if ( si == last )
				k = ( (unsigned long long)idx << 32 ) | (unsigned long long)(unsigned)v;
			kept.push_back( k );
		}
		std::sort( kept.begin(), kept.end() );
		if ( !kept.empty() )
			cudaMemcpyAsync( d.sensorPrevKeys, kept.data(), sizeof( unsigned long long ) * kept.size(),
							 cudaMemcpyHostToDevice, W->stream );
		int m = (int)kept.size();
		cudaMemcpyAsync( &d.sc->sensorPrev, &m, sizeof( int ), cudaMemcpyHostToDevice, W->stream );
		cudaStreamSynchronize( W->stream );
	}
	S[idx] = S[last];
	S.pop_back();
	W->sensorsDirty = true;
}

static void free_shape_host( HostWorld* W, int s )
{
	W->sflags[s] = 0;
	up( W->d.sflags, W->sflags, s, s + 1, W->stream );
	W->shapeFree.push_back( s );
}

// shape.c:230-316: out of the body's shape list, proxy, contacts (the body's
// contact list order), sensor, id
static void destroy_shape_host( HostWorld* W, int s, int wake )
{
	int b = W->shapeBody[s];
	if ( W->headShape[b] == s )
	{
		W->headShape[b] = W->nextShape[s];
		up( W->d.headShape, W->headShape, b, b + 1, W->stream );
	}
	else
		for ( int k = W->headShape[b]; k != F2D_NULL; k = W->nextShape[k] )
			if ( W->nextShape[k] == s )
			{
				W->nextShape[k] = W->nextShape[s];
				up( W->d.nextShape, W->nextShape, k, k + 1, W->stream );
				break;
			}
	destroy_proxy_host( W, s );
	launch_destroy_contacts_of( W->d, W->stream, b, s, -1, wake, W->s.tmpA );
	if ( W->sflags[s] & SF_SENSOR )
		destroy_sensor_host( W, s );
	free_shape_host( W, s );
}

static void destroy_chain_host( HostWorld* W, int c )
{
	int b = W->chainBody[c];
	if ( W->headChain[b] == c )
		W->headChain[b] = W->chainNext[c];
	else
		for ( int k = W->headChain[b]; k != F2D_NULL; k = W->chainNext[k] )
			if ( W->chainNext[k] == c )
			{
				W->chainNext[k] = W->chainNext[c];
				break;
			}
	for ( int s : W->chainSegments[c] )
		destroy_shape_host( W, s, 1 );
	W->chainSegments[c].clear();
	W->chainBody[c] = -1;
	W->chainFree.push_back( c );
}

// body.c:343-440: joints, contacts, shapes (sensors, proxies, ids), chains,
// island, solver set, id
static void destroy_body_host( HostWorld* W, int b )
{
	for ( int key = W->headJoint[b], g = 0; key != F2D_NULL && g <= W->jointCount; ++g )
	{
		int j = key >> 1;
		key = W->jnext[2 * j + ( key & 1 )];
		destroy_joint_host( W, j, 1 );
	}
	launch_destroy_contacts_of( W->d, W->stream, b, -1, -1, 1, W->s.tmpA );
	for ( int s = W->headShape[b]; s != F2D_NULL; s = W->nextShape[s] )
	{
		if ( W->sflags[s] & SF_SENSOR )
			destroy_sensor_host( W, s );
		destroy_proxy_host( W, s );
		free_shape_host( W, s );
	}
	for ( int c = W->headChain[b]; c != F2D_NULL; c = W->chainNext[c] )
	{
		W->chainSegments[c].clear();
		W->chainBody[c] = -1;
		W->chainFree.push_back( c );
	}
	W->headChain[b] = F2D_NULL;
	launch_destroy_body_records( W->d, W->stream, b );
	if ( !W->islOn && W->awakeSlot[b] >= 0 )
	{
		int k = W->awakeSlot[b];
		int m = W->awakeOrder.back();
		W->awakeOrder[k] = m;
		W->awakeSlot[m] = k;
		W->awakeOrder.pop_back();
		W->awakeSlot[b] = -1;
		W->awakeOrderDirty = true;
	}
	W->bflags[b] = 0;
	W->headShape[b] = F2D_NULL;
	W->headJoint[b] = F2D_NULL;
	W->jointCountB[b] = 0;
	up( W->d.headShape, W->headShape, b, b + 1, W->stream );
	up( W->d.headJoint, W->headJoint, b, b + 1, W->stream );
	up( W->d.jointCountB, W->jointCountB, b, b + 1, W->stream );
	W->bodyFree.push_back( b );
}

// RawBox2D.destroyBody (raw_box2d.dart:96) -> b2DestroyBody (body.c:343)
extern "C" F2D_API void f2d_destroy_body( int32_t index1, int32_t wg )
{
	HostWorld* W;
	int b = body_from( index1, wg, &W );
	if ( b < 0 )
		return;
	destroy_begin( W );
	destroy_body_host( W, b );
	destroy_end( W );
}

// RawBox2D.destroyShape (raw_box2d.dart:390) -> b2DestroyShape (shape.c:318)
extern "C" F2D_API void f2d_destroy_shape( int32_t index1, int32_t wg, int32_t updateBodyMass )
{
	HostWorld* W;
	int s = shape_from( index1, wg, &W );
	if ( s < 0 )
		return;
	int b = W->shapeBody[s];
	destroy_begin( W );
	destroy_shape_host( W, s, 1 );
	destroy_end( W );
	if ( updateBodyMass )
	{
		pull_body( W, b );
		update_mass( W, b );
		mark_body( W, b );
	}
}

// RawBox2D.destroyChain (raw_box2d.dart:550) -> b2DestroyChain (shape.c:488)
extern "C" F2D_API void f2d_destroy_chain( int32_t index1, int32_t wg )
{
	HostWorld* W = world_from_wg( wg );
	if ( W == nullptr || !chain_live( W, index1 - 1, wg ) )
		return;
	destroy_begin( W );
	destroy_chain_host( W, index1 - 1 );
	destroy_end( W );
}

// RawBox2D.destroyJoint (raw_box2d.dart:714) -> b2DestroyJoint (joint.c:808)
extern "C" F2D_API void f2d_destroy_joint( int32_t index1, int32_t wg )
{
	HostWorld* W = world_from_wg( wg );
	int j = index1 - 1;
	if ( W == nullptr || j < 0 || j >= W->jointCount || !joint_live( W, j, wg ) )
		return;
	destroy_begin( W );
	destroy_joint_host( W, j, 1 );
	destroy_end( W );
}

// joint.c:313-351 after a joint that keeps its bodies from colliding joined
// the graph: their contacts go, without waking (both contact lists hold the
// shared contacts in the same relative order, newest first)
static void destroy_contacts_between( HostWorld* W, int a, int b )
{
	if ( !W->stepped )
		return; // contacts exist only after a step
	destroy_begin( W );
	launch_destroy_contacts_of( W->d, W->stream, a, -1, b, 0, W->s.tmpA );
	destroy_end( W );
}

// RawBox2D.jointSetCollideConnected (b2Joint_SetCollideConnected,
// joint.c:980-1022): allowing collision buffers the proxies of the body with
// fewer shapes; forbidding it destroys the contacts between the bodies
extern "C" F2D_API void f2d_joint_set_collide_connected( int32_t index1, int32_t wg, int32_t flag )
{
	HostWorld* W = world_from_wg( wg );
	int j = index1 - 1;
	if ( W == nullptr || j < 0 || j >= W->jointCount || !joint_live( W, j, wg ) )
		return;
	bool on = flag != 0;
	if ( ( ( W->jflags[j] & JF_COLLIDE ) != 0 ) == on )
		return;
	W->jflags[j] = on ? ( W->jflags[j] | JF_COLLIDE ) : ( W->jflags[j] & ~JF_COLLIDE );
	mark_joint_dirty( W, j );
	int2 jb = W->jbody[j];
	if ( on )
	{
		auto count = [&]( int body ) {
			int n = 0;
			for ( int s = W->headShape[body]; s != F2D_NULL; s = W->nextShape[s] )
				n += 1;
			return n;
		};
		int body = count( jb.x ) < count( jb.y ) ? jb.x : jb.y;
		for ( int s = W->headShape[body]; s != F2D_NULL; s = W->nextShape[s] )
			if ( W->proxyKey[s] != F2D_NULL )
				host_move( W, s );
	}
	else
		destroy_contacts_between( W, jb.x, jb.y );
}

extern "C" F2D_API int32_t f2d_joint_get_collide_connected( int32_t index1, int32_t wg )
{
	HostWorld* W = world_from_wg( wg );
	int j = index1 - 1;
	if ( W == nullptr || j < 0 || j >= W->jointCount || !joint_live( W, j, wg ) )
		return 0;
	return ( W->jflags[j] & JF_COLLIDE ) != 0;
}

// ---------------------------------------------------------------------------
// properties: the RawBox2D getters and setters without a call of their own
// (bodies raw_box2d.dart:198-319, shapes :403-527, chains :553-569, joints
// :717-1285). Values the device changes (flags with dynamic bits, joint
// impulses) are edited in place on the stream; host-owned rows go up as
// single fields, so nothing the device keeps is overwritten.
// ---------------------------------------------------------------------------
__global__ void k_edit_bits( int* a, int i, int set, int clear )
{
	a[i] = ( a[i] & ~clear ) | set;
}

static void edit_body_bits( HostWorld* W, int b, int set, int clear )
{
	W->bflags[b] = ( W->bflags[b] & ~clear ) | set;
	if ( b < W->bodyUploaded )
		k_edit_bits<<<1, 1, 0, W->stream>>>( W->d.bflags, b, set, clear );
}

static void edit_shape_bits( HostWorld* W, int s, int set, int clear )
{
	W->sflags[s] = ( W->sflags[s] & ~clear ) | set;
	if ( s < W->shapeUploaded )
		k_edit_bits<<<1, 1, 0, W->stream>>>( W->d.sflags, s, set, clear );
}

static fxf body_xf( HostWorld* W, int b )
{
	pull_body( W, b );
	float4 x = W->xf[b];
	fxf t;
	t.p = mk( x.x, x.y );
	t.q.c = x.z;
	t.q.s = x.w;
	return t;
}

// ---------------------------------------------------------------------------
// body type, disable and enable (body.c:1036-1282, 1557-1700): contacts and
// proxies on the host side of the boundary as the destroy path does them,
// solver sets, islands and graph colours in one device launch each
// ---------------------------------------------------------------------------
// the awake set's body array of a world without islands
static void awake_order_add( HostWorld* W, int b )
{
	if ( W->islOn || W->awakeSlot[b] >= 0 )
		return;
	W->awakeSlot[b] = (int)W->awakeOrder.size();
	W->awakeOrder.push_back( b );
	W->awakeOrderDirty = true;
}

static void awake_order_remove( HostWorld* W, int b )
{
	if ( W->islOn || W->awakeSlot[b] < 0 )
		return;
	int k = W->awakeSlot[b];
	int m = W->awakeOrder.back();
	W->awakeOrder[k] = m;
	W->awakeSlot[m] = k;
	W->awakeOrder.pop_back();
	W->awakeSlot[b] = -1;
	W->awakeOrderDirty = true;
}

// shape.c:585-601 b2CreateShapeProxy with forcePairCreation: the boxes for
// the proxy's type, a leaf of that tree, the proxy buffered as moved
static void create_proxy_forced( HostWorld* W, int s, int proxyType )
{
	int b = W->shapeBody[s];
	fxf xf = body_xf( W, b );
	fbox aabb = box_grow( h_shape_aabb( W->hgeomv[s], xf ), F2D_SPECULATIVE );
	fbox fat = box_grow( aabb, proxyType == 0 ? F2D_SPECULATIVE : F2D_AABB_MARGIN );
	W->aabb[s] = box_to4( aabb );
	W->fat[s] = box_to4( fat );
	tree_pull( W, proxyType );
	int proxyId = W->trees[proxyType].create_proxy( W->fat[s], W->cat[s], s );
	W->treeDirty[proxyType] = true;
	if ( proxyType == 0 )
		W->staticDirty = true;
	W->proxyKey[s] = ( proxyId << 2 ) | proxyType;
	if ( s < W->shapeUploaded )
	{
		up( W->d.proxyKey, W->proxyKey, s, s + 1, W->stream );
		up( W->d.aabb, W->aabb, s, s + 1, W->stream );
		up( W->d.fat, W->fat, s, s + 1, W->stream );
	}
	host_move( W, s );
}

// after the device launch: the body's rows (type, state, flags) come back
// to the host mirror, then its mass data (b2UpdateBodyMassData)
static void type_change_end( HostWorld* W, int b )
{
	destroy_end( W );
	body_rows_changed( W, false );
	pull_body( W, b );
	update_mass( W, b );
	mark_body( W, b );
}

// RawBox2D.bodySetType (raw_box2d.dart:220) -> b2Body_SetType (body.c:1036)
extern "C" F2D_API void f2d_body_set_type( int32_t index1, int32_t wg, int32_t type )
{
	HostWorld* W;
	int b = body_from( index1, wg, &W );
	if ( b < 0 || type < 0 || type > 2 )
		return;
	pull_body( W, b );
	int f = W->bflags[b];
	int orig = body_type( f );
	if ( orig == type )
		return;
	if ( ( f & BF_ENABLED ) == 0 )
	{
		// a disabled body changes no set, island or proxy
		edit_body_bits( W, b, type << BF_TYPE_SHIFT, 3 << BF_TYPE_SHIFT );
		update_mass( W, b );
		mark_body( W, b );
		return;
	}
	destroy_begin( W );
	launch_destroy_contacts_of( W->d, W->stream, b, -1, -1, 0, W->s.tmpA );
	launch_body_set_type( W->d, W->stream, b, type );
	W->bflags[b] = ( f & ~( 3 << BF_TYPE_SHIFT ) ) | ( type << BF_TYPE_SHIFT );
	if ( orig == 0 )
		awake_order_add( W, b );
	else if ( type == 0 )
		awake_order_remove( W, b );
	for ( int s = W->headShape[b]; s != F2D_NULL; s = W->nextShape[s] )
	{
		destroy_proxy_host( W, s );
		create_proxy_forced( W, s, type );
	}
	type_change_end( W, b );
}

// RawBox2D.bodyDisable (raw_box2d.dart:254) -> b2Body_Disable (body.c:1557)
extern "C" F2D_API void f2d_body_disable( int32_t index1, int32_t wg )
{
	HostWorld* W;
	int b = body_from( index1, wg, &W );
	if ( b < 0 )
		return;
	pull_body( W, b );
	if ( ( W->bflags[b] & BF_ENABLED ) == 0 )
		return;
	destroy_begin( W );
	launch_destroy_contacts_of( W->d, W->stream, b, -1, -1, 1, W->s.tmpA );
	for ( int s = W->headShape[b]; s != F2D_NULL; s = W->nextShape[s] )
	{
		destroy_proxy_host( W, s );
		edit_shape_bits( W, s, 0, SF_PROXY );
	}
	launch_body_disable( W->d, W->stream, b );
	W->bflags[b] &= ~( BF_ENABLED | BF_ASLEEP );
	awake_order_remove( W, b );
	type_change_end( W, b );
}

// RawBox2D.bodyEnable (raw_box2d.dart:258) -> b2Body_Enable (body.c:1628)
extern "C" F2D_API void f2d_body_enable( int32_t index1, int32_t wg )
{
	HostWorld* W;
	int b = body_from( index1, wg, &W );
	if ( b < 0 )
		return;
	pull_body( W, b );
	int f = W->bflags[b];
	if ( f & BF_ENABLED )
		return;
	destroy_begin( W );
	launch_body_enable( W->d, W->stream, b );
	W->bflags[b] = f | BF_ENABLED;
	int type = body_type( f );
	if ( type != 0 )
		awake_order_add( W, b );
	for ( int s = W->headShape[b]; s != F2D_NULL; s = W->nextShape[s] )
	{
		create_proxy_forced( W, s, type );
		edit_shape_bits( W, s, SF_PROXY, 0 );
	}
	type_change_end( W, b );
}

extern "C" F2D_API double f2d_body_get_param( int32_t index1, int32_t wg, int32_t code )
{
	HostWorld* W;
	int b = body_from( index1, wg, &W );
	if ( b < 0 )
		return 0.0;
	pull_body( W, b );
	int f = W->bflags[b];
	switch ( code )
	{
		case F2D_BODY_LINEAR_DAMPING:
			return W->damp[b].x;
		case F2D_BODY_ANGULAR_DAMPING:
			return W->damp[b].y;
		case F2D_BODY_GRAVITY_SCALE:
			return W->damp[b].z;
		case F2D_BODY_BULLET:
			return ( f & BF_BULLET ) != 0;
		case F2D_BODY_FIXED_ROTATION:
			return ( f & BF_FIXED_ROT ) != 0;
		case F2D_BODY_ENABLED:
			return ( f & BF_ENABLED ) != 0;
		case F2D_BODY_TYPE:
			return body_type( f );
		case F2D_BODY_LOCAL_CENTER_X:
			return W->localCenter[b].x;
		case F2D_BODY_LOCAL_CENTER_Y:
			return W->localCenter[b].y;
		case F2D_BODY_WORLD_CENTER_X:
			return W->center[b].x;
		case F2D_BODY_WORLD_CENTER_Y:
			return W->center[b].y;
		default:
			return 0.0;
	}
}

// body.c:1412-1480 (damping, gravity scale: the value only), :1560-1580
// (bullet), :1536-1558 (fixed rotation: angular velocity cleared, mass
// recomputed)
extern "C" F2D_API void f2d_body_set_param( int32_t index1, int32_t wg, int32_t code, double value )
{
	HostWorld* W;
	int b = body_from( index1, wg, &W );
	if ( b < 0 )
		return;
	float v = (float)value;
	auto damp = [&]( int k ) {
		float4& d = W->damp[b];
		( k == 0 ? d.x : k == 1 ? d.y : d.z ) = v;
		if ( b < W->bodyUploaded )
			up( W->d.damp, W->damp, b, b + 1, W->stream );
	};
	switch ( code )
	{
		case F2D_BODY_LINEAR_DAMPING:
			if ( valid_float( value ) && value >= 0.0 )
				damp( 0 );
			break;
		case F2D_BODY_ANGULAR_DAMPING:
			if ( valid_float( value ) && value >= 0.0 )
				damp( 1 );
			break;
		case F2D_BODY_GRAVITY_SCALE:
			if ( valid_float( value ) )
				damp( 2 );
			break;
		case F2D_BODY_BULLET:
			edit_body_bits( W, b, value != 0.0 ? BF_BULLET : 0, value != 0.0 ? 0 : BF_BULLET );
			break;
		case F2D_BODY_FIXED_ROTATION:
		{
			bool on = value != 0.0;
			if ( ( ( W->bflags[b] & BF_FIXED_ROT ) != 0 ) == on )
				break;
			pull_body( W, b );
			W->bflags[b] = on ? ( W->bflags[b] | BF_FIXED_ROT ) : ( W->bflags[b] & ~BF_FIXED_ROT );
			W->vel[b].z = 0.0f;
			update_mass( W, b );
			mark_body( W, b );
			break;
		}
		default:
			break;
	}
}

extern "C" F2D_API void f2d_body_get_world_point( int32_t index1, int32_t wg, double x, double y, double* ox,
												  double* oy )
{
	*ox = *oy = 0.0;
	HostWorld* W;
	int b = body_from( index1, wg, &W );
	if ( b < 0 )
		return;
	fv2 p = xpoint( body_xf( W, b ), mk( (float)x, (float)y ) );
	*ox = p.x;
	*oy = p.y;
}

extern "C" F2D_API void f2d_body_get_local_point( int32_t index1, int32_t wg, double x, double y, double* ox,
												  double* oy )
{
	*ox = *oy = 0.0;
	HostWorld* W;
	int b = body_from( index1, wg, &W );
	if ( b < 0 )
		return;
	fxf t = body_xf( W, b );
	fv2 p = rinvrot( t.q, vsub( mk( (float)x, (float)y ), t.p ) );
	*ox = p.x;
	*oy = p.y;
}

// body.c:1357-1381: mass, inertia and local centre as given (extents kept)
extern "C" F2D_API void f2d_body_set_mass_data( int32_t index1, int32_t wg, double mass, double rotationalInertia,
												double centerX, double centerY )
{
	HostWorld* W;
	int b = body_from( index1, wg, &W );
	if ( b < 0 || !valid_float( mass ) || mass < 0.0 || !valid_float( rotationalInertia ) || rotationalInertia < 0.0 ||
		 !valid_float( centerX ) || !valid_float( centerY ) )
		return;
	fxf t = body_xf( W, b );
	float m = (float)mass, I = (float)rotationalInertia;
	fv2 lc = mk( (float)centerX, (float)centerY );
	fv2 c = xpoint( t, lc );
	W->bmass[b] = m;
	W->binertia[b] = I;
	W->localCenter[b] = make_float2( lc.x, lc.y );
	W->center[b] = make_float2( c.x, c.y );
	float4 s0 = W->sweep0[b];
	W->sweep0[b] = make_float4( c.x, c.y, s0.z, s0.w );
	float4 mv = W->massv[b];
	W->massv[b] = make_float4( m > 0.0f ? 1.0f / m : 0.0f, I > 0.0f ? 1.0f / I : 0.0f, mv.z, mv.w );
	mark_body( W, b );
}

extern "C" F2D_API void f2d_body_apply_mass_from_shapes( int32_t index1, int32_t wg )
{
	HostWorld* W;
	int b = body_from( index1, wg, &W );
	if ( b < 0 )
		return;
	pull_body( W, b );
	update_mass( W, b );
	mark_body( W, b );
}

extern "C" F2D_API void f2d_body_set_name( int32_t index1, int32_t wg, const char* name )
{
	HostWorld* W;
	int b = body_from( index1, wg, &W );
	if ( b < 0 )
		return;
	if ( (int)W->bname.size() <= b )
		W->bname.resize( (size_t)b + 1 );
	std::string& n = W->bname[b];
	n.clear();
	if ( name != nullptr )
		for ( int i = 0; i < 31 && name[i] != 0; ++i )
			n.push_back( name[i] );
}

extern "C" F2D_API int32_t f2d_body_get_name( int32_t index1, int32_t wg, char* out, int32_t capacity )
{
	HostWorld* W;
	int b = body_from( index1, wg, &W );
	if ( out && capacity > 0 )
		out[0] = 0;
	if ( b < 0 || b >= (int)W->bname.size() )
		return 0;
	const std::string& n = W->bname[b];
	if ( out && capacity > 0 )
	{
		int k = std::min( (int)n.size(), capacity - 1 );
		memcpy( out, n.data(), (size_t)k );
		out[k] = 0;
	}
	return (int32_t)n.size();
}

extern "C" F2D_API int32_t f2d_body_get_shapes( int32_t index1, int32_t wg, int32_t* out2, int32_t capacity )
{
	HostWorld* W;
	int b = body_from( index1, wg, &W );
	if ( b < 0 )
		return 0;
	int n = 0;
	for ( int s = W->headShape[b]; s != F2D_NULL; s = W->nextShape[s], ++n )
		if ( out2 && n < capacity )
		{
			out2[2 * n] = s + 1;
			out2[2 * n + 1] = pack_wg( W, W->sgen[s] );
		}
	return n;
}

extern "C" F2D_API int32_t f2d_body_get_joints( int32_t index1, int32_t wg, int32_t* out2, int32_t capacity )
{
	HostWorld* W;
	int b = body_from( index1, wg, &W );
	if ( b < 0 )
		return 0;
	int n = 0;
	for ( int key = W->headJoint[b]; key != F2D_NULL && n <= W->jointCount; key = W->jnext[2 * ( key >> 1 ) + ( key & 1 )], ++n )
		if ( out2 && n < capacity )
		{
			int j = key >> 1;
			out2[2 * n] = j + 1;
			out2[2 * n + 1] = pack_wg( W, W->jgen[j] );
		}
	return n;
}

extern "C" F2D_API double f2d_shape_get_param( int32_t index1, int32_t wg, int32_t code )
{
	HostWorld* W;
	int s = shape_from( index1, wg, &W );
	if ( s < 0 )
		return 0.0;
	int f = W->sflags[s];
	switch ( code )
	{
		case F2D_SHAPE_DENSITY:
			return W->density[s];
		case F2D_SHAPE_FRICTION:
			return W->mat[s].x;
		case F2D_SHAPE_RESTITUTION:
			return W->mat[s].y;
		case F2D_SHAPE_SENSOR:
			return ( f & SF_SENSOR ) != 0;
		case F2D_SHAPE_SENSOR_EVENTS:
			return ( f & SF_SENSOR_EVENTS ) != 0;
		case F2D_SHAPE_CONTACT_EVENTS:
			return ( f & SF_CONTACT_EVENTS ) != 0;
		case F2D_SHAPE_HIT_EVENTS:
			return ( f & SF_HIT_EVENTS ) != 0;
		case F2D_SHAPE_PRESOLVE_EVENTS:
			return ( f & SF_PRESOLVE ) != 0;
		case F2D_SHAPE_CATEGORY:
			return (double)(int64_t)W->cat[s];
		case F2D_SHAPE_MASK:
			return (double)(int64_t)W->mask[s];
		case F2D_SHAPE_GROUP:
			return W->group[s];
		default:
			return 0.0;
	}
}

// shape.c:1057-1183: density (mass recomputed on request), friction and
// restitution (mixed into the contacts at their next update), event flags
// (read when contacts are created, hit and sensor flags every step)
static void shape_set( HostWorld* W, int s, int code, double value, int flag )
{
	float v = (float)value;
	int bit = code == F2D_SHAPE_SENSOR_EVENTS	 ? SF_SENSOR_EVENTS
			  : code == F2D_SHAPE_CONTACT_EVENTS ? SF_CONTACT_EVENTS
			  : code == F2D_SHAPE_HIT_EVENTS	 ? SF_HIT_EVENTS
			  : code == F2D_SHAPE_PRESOLVE_EVENTS ? SF_PRESOLVE
												  : 0;
	if ( bit )
	{
		edit_shape_bits( W, s, value != 0.0 ? bit : 0, value != 0.0 ? 0 : bit );
		return;
	}
	switch ( code )
	{
		case F2D_SHAPE_DENSITY:
		{
			if ( !valid_float( value ) || value < 0.0 || v == W->density[s] )
				return;
			W->density[s] = v;
			if ( flag )
			{
				int b = W->shapeBody[s];
				pull_body( W, b );
				update_mass( W, b );
				mark_body( W, b );
			}
			return;
		}
		case F2D_SHAPE_FRICTION:
		case F2D_SHAPE_RESTITUTION:
			if ( !valid_float( value ) || value < 0.0 )
				return;
			( code == F2D_SHAPE_FRICTION ? W->mat[s].x : W->mat[s].y ) = v;
			if ( s < W->shapeUploaded )
				up( W->d.mat, W->mat, s, s + 1, W->stream );
			return;
		default:
			return;
	}
}

extern "C" F2D_API void f2d_shape_set_param( int32_t index1, int32_t wg, int32_t code, double value, int32_t flag )
{
	HostWorld* W;
	int s = shape_from( index1, wg, &W );
	if ( s >= 0 )
		shape_set( W, s, code, value, flag );
}

extern "C" F2D_API int32_t f2d_shape_get_body( int32_t index1, int32_t wg, int32_t* bodyIndex1, int32_t* bodyWg )
{
	*bodyIndex1 = *bodyWg = 0;
	HostWorld* W;
	int s = shape_from( index1, wg, &W );
	if ( s < 0 )
		return 0;
	int b = W->shapeBody[s];
	*bodyIndex1 = b + 1;
	*bodyWg = pack_wg( W, W->bgen[b] );
	return 1;
}

// shape.c:1185-1262 b2Shape_SetFilter / b2ResetProxy: the shape's contacts
// end (waking), its boxes are recomputed; a new category re-creates the
// proxy (new node, forced pair search), otherwise the proxy moves
extern "C" F2D_API void f2d_shape_set_filter( int32_t index1, int32_t wg, int64_t categoryBits, int64_t maskBits,
											  int32_t groupIndex )
{
	HostWorld* W;
	int s = shape_from( index1, wg, &W );
	if ( s < 0 )
		return;
	unsigned long long cat = (unsigned long long)categoryBits, mask = (unsigned long long)maskBits;
	if ( cat == W->cat[s] && mask == W->mask[s] && groupIndex == W->group[s] )
		return;
	bool destroyProxy = cat != W->cat[s];
	W->cat[s] = cat;
	W->mask[s] = mask;
	W->group[s] = groupIndex;
	int b = W->shapeBody[s];
	destroy_begin( W );
	launch_destroy_contacts_of( W->d, W->stream, b, s, -1, 1, W->s.tmpA );
	if ( s < W->shapeUploaded )
	{
		up( W->d.cat, W->cat, s, s + 1, W->stream );
		up( W->d.mask, W->mask, s, s + 1, W->stream );
		up( W->d.group, W->group, s, s + 1, W->stream );
	}
	fxf xf = body_xf( W, b );
	int pk = W->proxyKey[s];
	int proxyType = pk != F2D_NULL ? ( pk & 3 ) : body_type( W->bflags[b] );
	fbox aabb = box_grow( h_shape_aabb( W->hgeomv[s], xf ), F2D_SPECULATIVE );
	fbox fat = box_grow( aabb, proxyType == 0 ? F2D_SPECULATIVE : F2D_AABB_MARGIN );
	W->aabb[s] = box_to4( aabb );
	W->fat[s] = box_to4( fat );
	if ( pk != F2D_NULL )
	{
		int t = pk & 3;
		tree_pull( W, t );
		if ( destroyProxy )
		{
			launch_unbuffer_move( W->d, W->stream, s );
			W->trees[t].destroy_proxy( pk >> 2 );
			int proxyId = W->trees[t].create_proxy( W->fat[s], cat, s );
			W->proxyKey[s] = ( proxyId << 2 ) | t;
			if ( s < W->shapeUploaded )
				up( W->d.proxyKey, W->proxyKey, s, s + 1, W->stream );
		}
		else
			W->trees[t].move_proxy( pk >> 2, W->fat[s] );
		W->treeDirty[t] = true;
		if ( t == 0 )
			W->staticDirty = true;
		host_move( W, s );
	}
	if ( s < W->shapeUploaded )
	{
		up( W->d.aabb, W->aabb, s, s + 1, W->stream );
		up( W->d.fat, W->fat, s, s + 1, W->stream );
	}
	destroy_end( W );
}

extern "C" F2D_API int32_t f2d_shape_test_point( int32_t index1, int32_t wg, double x, double y )
{
	HostWorld* W;
	int s = shape_from( index1, wg, &W );
	if ( s < 0 )
		return 0;
	flush_uploads( W );
	int* dOut = W->s.tmpA;
	launch_shape_test_point( W->d, W->stream, s, (float)x, (float)y, dOut );
	int r = 0;
	cudaMemcpyAsync( &r, dOut, sizeof( int ), cudaMemcpyDeviceToHost, W->stream );
	cudaStreamSynchronize( W->stream );
	return r;
}

extern "C" F2D_API int32_t f2d_shape_get_geometry( int32_t index1, int32_t wg, int32_t type, double* out,
												   int32_t capacity )
{
	HostWorld* W;
	int s = shape_from( index1, wg, &W );
	if ( s < 0 )
		return 0;
	const HShapeGeom& g = W->hgeomv[s];
	if ( g.type != type )
		return 0;
	double v[2 * F2D_MAX_POLY + 1];
	int n = 0;
	switch ( g.type )
	{
		case ST_CIRCLE:
			v[n++] = g.c1.x, v[n++] = g.c1.y, v[n++] = g.radius;
			break;
		case ST_CAPSULE:
			v[n++] = g.c1.x, v[n++] = g.c1.y, v[n++] = g.c2.x, v[n++] = g.c2.y, v[n++] = g.radius;
			break;
		case ST_SEGMENT:
		case ST_CHAIN:
			v[n++] = g.c1.x, v[n++] = g.c1.y, v[n++] = g.c2.x, v[n++] = g.c2.y;
			break;
		case ST_POLYGON:
			for ( int i = 0; i < g.poly.count; ++i )
				v[n++] = g.poly.v[i].x, v[n++] = g.poly.v[i].y;
			v[n++] = g.poly.radius;
			break;
		default:
			return 0;
	}
	for ( int i = 0; i < n && i < capacity; ++i )
		out[i] = v[i];
	return n;
}

extern "C" F2D_API void f2d_shape_get_aabb( int32_t index1, int32_t wg, double* out4 )
{
	out4[0] = out4[1] = out4[2] = out4[3] = 0.0;
	HostWorld* W;
	int s = shape_from( index1, wg, &W );
	if ( s < 0 )
		return;
	flush_uploads( W );
	cudaStreamSynchronize( W->stream );
	float4 a;
	cudaMemcpy( &a, W->d.aabb + s, sizeof( float4 ), cudaMemcpyDeviceToHost );
	out4[0] = a.x;
	out4[1] = a.y;
	out4[2] = a.z;
	out4[3] = a.w;
}

extern "C" F2D_API int32_t f2d_chain_is_valid( int32_t index1, int32_t wg )
{
	HostWorld* W = world_from_wg( wg );
	return W != nullptr && chain_live( W, index1 - 1, wg );
}

// shape.c:1476-1530: the chain's materials and every segment
extern "C" F2D_API double f2d_chain_get_param( int32_t index1, int32_t wg, int32_t code )
{
	HostWorld* W = world_from_wg( wg );
	if ( W == nullptr || !chain_live( W, index1 - 1, wg ) )
		return 0.0;
	int s = W->chainSegments[index1 - 1].front();
	return code == F2D_SHAPE_FRICTION ? W->mat[s].x : code == F2D_SHAPE_RESTITUTION ? W->mat[s].y : 0.0;
}

extern "C" F2D_API void f2d_chain_set_param( int32_t index1, int32_t wg, int32_t code, double value )
{
	HostWorld* W = world_from_wg( wg );
	if ( W == nullptr || !chain_live( W, index1 - 1, wg ) )
		return;
	if ( code != F2D_SHAPE_FRICTION && code != F2D_SHAPE_RESTITUTION )
		return;
	for ( int s : W->chainSegments[index1 - 1] )
		shape_set( W, s, code, value, 0 );
}

// joint rows by type (the layouts beside the solvers in joint.cuh)
static float* joint_field( HostWorld* W, int j, int type, int code )
{
	float4& d0 = W->jdef0[j];
	float4& d1 = W->jdef1[j];
	float4& d2 = W->jdef2[j];
	float4& d3 = W->jdef3[j];
	switch ( code )
	{
		case F2D_JP_LOCAL_ANCHOR_AX:
			return &d0.x;
		case F2D_JP_LOCAL_ANCHOR_AY:
			return &d0.y;
		case F2D_JP_LOCAL_ANCHOR_BX:
			return &d0.z;
		case F2D_JP_LOCAL_ANCHOR_BY:
			return &d0.w;
		default:
			break;
	}
	switch ( type )
	{
		case 0: // revolute
			switch ( code )
			{
				case F2D_JP_SPRING_HERTZ: return &d1.z;
				case F2D_JP_SPRING_DAMPING: return &d1.w;
				case F2D_JP_TARGET: return &d1.y;
				case F2D_JP_LOWER: return &d2.x;
				case F2D_JP_UPPER: return &d2.y;
				case F2D_JP_MAX_MOTOR: return &d2.z;
				case F2D_JP_MOTOR_SPEED: return &d2.w;
			}
			break;
		case F2D_JOINT_PRISMATIC:
			switch ( code )
			{
				case F2D_JP_SPRING_HERTZ: return &d3.x;
				case F2D_JP_SPRING_DAMPING: return &d3.y;
				case F2D_JP_TARGET: return &d1.w;
				case F2D_JP_LOWER: return &d2.x;
				case F2D_JP_UPPER: return &d2.y;
				case F2D_JP_MAX_MOTOR: return &d2.z;
				case F2D_JP_MOTOR_SPEED: return &d2.w;
			}
			break;
		case F2D_JOINT_WHEEL:
			switch ( code )
			{
				case F2D_JP_SPRING_HERTZ: return &d1.z;
				case F2D_JP_SPRING_DAMPING: return &d1.w;
				case F2D_JP_LOWER: return &d2.x;
				case F2D_JP_UPPER: return &d2.y;
				case F2D_JP_MAX_MOTOR: return &d2.z;
				case F2D_JP_MOTOR_SPEED: return &d2.w;
			}
			break;
		case F2D_JOINT_DISTANCE:
			switch ( code )
			{
				case F2D_JP_LENGTH: return &d1.x;
				case F2D_JP_MIN_LENGTH: return &d1.y;
				case F2D_JP_MAX_LENGTH: return &d1.z;
				case F2D_JP_SPRING_HERTZ: return &d1.w;
				case F2D_JP_SPRING_DAMPING: return &d2.x;
				case F2D_JP_MAX_MOTOR: return &d2.y;
				case F2D_JP_MOTOR_SPEED: return &d2.z;
			}
			break;
		case F2D_JOINT_WELD:
			switch ( code )
			{
				case F2D_JP_LINEAR_HERTZ: return &d1.y;
				case F2D_JP_LINEAR_DAMPING: return &d1.z;
				case F2D_JP_ANGULAR_HERTZ: return &d1.w;
				case F2D_JP_ANGULAR_DAMPING: return &d2.x;
			}
			break;
		case F2D_JOINT_MOTOR:
			switch ( code )
			{
				case F2D_JP_LINEAR_OFFSET_X: return &d1.x;
				case F2D_JP_LINEAR_OFFSET_Y: return &d1.y;
				case F2D_JP_ANGULAR_OFFSET: return &d1.z;
				case F2D_JP_MAX_FORCE: return &d1.w;
				case F2D_JP_MAX_TORQUE: return &d2.x;
				case F2D_JP_CORRECTION: return &d2.y;
			}
			break;
		case F2D_JOINT_MOUSE:
			switch ( code )
			{
				case F2D_JP_TARGET_X: return &d1.x;
				case F2D_JP_TARGET_Y: return &d1.y;
				case F2D_JP_SPRING_HERTZ: return &d1.z;
				case F2D_JP_SPRING_DAMPING: return &d1.w;
				case F2D_JP_MAX_FORCE: return &d2.x;
			}
			break;
	}
	return nullptr;
}

// the flag bit a code switches, for the types that have it
static int joint_bit( int type, int code )
{
	bool sprung = type == 0 || type == F2D_JOINT_PRISMATIC || type == F2D_JOINT_WHEEL || type == F2D_JOINT_DISTANCE;
	if ( !sprung )
		return 0;
	return code == F2D_JP_SPRING_ENABLED ? JF_SPRING
		   : code == F2D_JP_LIMIT_ENABLED ? JF_LIMIT
		   : code == F2D_JP_MOTOR_ENABLED ? JF_MOTOR
										  : 0;
}

// b2JointType values (types.h:630-640) of the library's joint types
static int reference_joint_type( int type )
{
	switch ( type )
	{
		case F2D_JOINT_DISTANCE: return 0;
		case F2D_JOINT_FILTER: return 1;
		case F2D_JOINT_MOTOR: return 2;
		case F2D_JOINT_MOUSE: return 3;
		case F2D_JOINT_PRISMATIC: return 4;
		case 0: return 5;
		case F2D_JOINT_WELD: return 6;
		case F2D_JOINT_WHEEL: return 7;
		default: return -1;
	}
}

static float4 joint_impulses( HostWorld* W, int j, float2* imp2 )
{
	float4 imp = make_float4( 0.0f, 0.0f, 0.0f, 0.0f );
	*imp2 = make_float2( 0.0f, 0.0f );
	if ( j < W->jointUploaded )
	{
		cudaStreamSynchronize( W->stream );
		cudaMemcpy( &imp, W->d.jimp + j, sizeof( imp ), cudaMemcpyDeviceToHost );
		cudaMemcpy( imp2, W->d.jimp2 + j, sizeof( float2 ), cudaMemcpyDeviceToHost );
	}
	return imp;
}

extern "C" F2D_API double f2d_joint_get_param( int32_t index1, int32_t wg, int32_t code )
{
	HostWorld* W = world_from_wg( wg );
	int j = index1 - 1;
	if ( W == nullptr || j < 0 || j >= W->jointCount || !joint_live( W, j, wg ) )
		return 0.0;
	int type = ( W->jflags[j] >> JF_TYPE_SHIFT ) & 0xf;
	if ( code == F2D_JP_TYPE )
		return reference_joint_type( type );
	if ( int bit = joint_bit( type, code ) )
		return ( W->jflags[j] & bit ) != 0;
	int a = W->jbody[j].x, b = W->jbody[j].y;
	float4 d0 = W->jdef0[j];
	if ( code == F2D_JP_MOTOR_EFFORT )
	{
		float2 imp2;
		float4 imp = joint_impulses( W, j, &imp2 );
		// revolute_joint.c:157, prismatic_joint.c:152, distance_joint.c:175
		// (motor impulse in w), wheel_joint.c:142 (in z)
		if ( type == 0 || type == F2D_JOINT_PRISMATIC || type == F2D_JOINT_DISTANCE )
			return W->invH * imp.w;
		if ( type == F2D_JOINT_WHEEL )
			return W->invH * imp.z;
		return 0.0;
	}
	if ( code == F2D_JP_CURRENT )
	{
		fxf ta = body_xf( W, a ), tb = body_xf( W, b );
		if ( type == 0 ) // revolute_joint.c:72-82
			return remainderf( relative_angle( tb.q, ta.q ) - W->jdef1[j].x, 2.0f * F2D_PI );
		if ( type == F2D_JOINT_DISTANCE ) // distance_joint.c:79-98
			return vlen( vsub( xpoint( tb, mk( d0.z, d0.w ) ), xpoint( ta, mk( d0.x, d0.y ) ) ) );
		if ( type == F2D_JOINT_PRISMATIC ) // prismatic_joint.c:158-172
		{
			fv2 axisA = rrot( ta.q, mk( W->jdef1[j].x, W->jdef1[j].y ) );
			fv2 d = vsub( xpoint( tb, mk( d0.z, d0.w ) ), xpoint( ta, mk( d0.x, d0.y ) ) );
			return vdot( d, axisA );
		}
		return 0.0;
	}
	if ( code == F2D_JP_SPEED && type == F2D_JOINT_PRISMATIC ) // prismatic_joint.c:174-209
	{
		fxf ta = body_xf( W, a ), tb = body_xf( W, b );
		fv2 axisA = rrot( ta.q, mk( W->jdef1[j].x, W->jdef1[j].y ) );
		fv2 cA = mk( W->center[a].x, W->center[a].y ), cB = mk( W->center[b].x, W->center[b].y );
		fv2 rA = rrot( ta.q, vsub( mk( d0.x, d0.y ), mk( W->localCenter[a].x, W->localCenter[a].y ) ) );
		fv2 rB = rrot( tb.q, vsub( mk( d0.z, d0.w ), mk( W->localCenter[b].x, W->localCenter[b].y ) ) );
		fv2 d = vadd( vsub( cB, cA ), vsub( rB, rA ) );
		// a body outside the awake set has no state: zero velocity
		auto moving = [&]( int body ) {
			int f = W->bflags[body];
			return body_type( f ) != 0 && ( f & BF_ENABLED ) && ( f & BF_ASLEEP ) == 0;
		};
		fv2 vA = moving( a ) ? mk( W->vel[a].x, W->vel[a].y ) : mk( 0.0f, 0.0f );
		fv2 vB = moving( b ) ? mk( W->vel[b].x, W->vel[b].y ) : mk( 0.0f, 0.0f );
		float wA = moving( a ) ? W->vel[a].z : 0.0f;
		float wB = moving( b ) ? W->vel[b].z : 0.0f;
		fv2 vRel = vsub( vadd( vB, vcrossSV( wB, rB ) ), vadd( vA, vcrossSV( wA, rA ) ) );
		return vdot( d, vcrossSV( wA, axisA ) ) + vdot( axisA, vRel );
	}
	float* f = joint_field( W, j, type, code );
	return f ? *f : 0.0;
}

// zero impulse components of joint j on the device (stream-ordered): mask
// bits 0-3 the jimp components, 4-5 the jimp2 components
static void clear_joint_impulses( HostWorld* W, int j, int mask )
{
	if ( j >= W->jointUploaded )
		return;
	for ( int k = 0; k < 4; ++k )
		if ( mask & ( 1 << k ) )
			cudaMemsetAsync( (float*)( W->d.jimp + j ) + k, 0, sizeof( float ), W->stream );
	for ( int k = 0; k < 2; ++k )
		if ( mask & ( 16 << k ) )
			cudaMemsetAsync( (float*)( W->d.jimp2 + j ) + k, 0, sizeof( float ), W->stream );
}

// revolute_joint.c:29-168, prismatic_joint.c:27-156, wheel_joint.c:27-145,
// distance_joint.c:27-178, weld_joint.c:19-63, motor_joint.c:19-73,
// mouse_joint.c:20-63: the value (clamped where the setter clamps); the
// impulses the setter clears
extern "C" F2D_API void f2d_joint_set_param( int32_t index1, int32_t wg, int32_t code, double value, double value2 )
{
	HostWorld* W = world_from_wg( wg );
	int j = index1 - 1;
	if ( W == nullptr || j < 0 || j >= W->jointCount || !joint_live( W, j, wg ) )
		return;
	int type = ( W->jflags[j] >> JF_TYPE_SHIFT ) & 0xf;
	float v = (float)value, v2 = (float)value2;
	// components of jimp (bits 0-3) and jimp2 (bits 4-5) per impulse kind
	int springImp = type == F2D_JOINT_WHEEL ? 2 : 4;
	int motorImp = type == F2D_JOINT_WHEEL ? 4 : 8;
	int limitImp = type == F2D_JOINT_DISTANCE ? 0 : 48;
	if ( int bit = joint_bit( type, code ) )
	{
		bool on = value != 0.0;
		if ( ( ( W->jflags[j] & bit ) != 0 ) == on )
			return;
		W->jflags[j] ^= bit;
		if ( bit == JF_SPRING && type != F2D_JOINT_DISTANCE )
			clear_joint_impulses( W, j, springImp );
		else if ( bit == JF_LIMIT )
			clear_joint_impulses( W, j, limitImp );
		else if ( bit == JF_MOTOR )
			clear_joint_impulses( W, j, motorImp );
		mark_joint_dirty( W, j );
		return;
	}
	if ( code == F2D_JP_LOWER && ( type == 0 || type == F2D_JOINT_PRISMATIC || type == F2D_JOINT_WHEEL ) )
	{
		float4& d2 = W->jdef2[j];
		if ( v != d2.x || v2 != d2.y )
		{
			d2.x = fmin_s( v, v2 );
			d2.y = fmax_s( v, v2 );
			clear_joint_impulses( W, j, 48 );
			mark_joint_dirty( W, j );
		}
		return;
	}
	if ( type == F2D_JOINT_DISTANCE && ( code == F2D_JP_LENGTH || code == F2D_JP_MIN_LENGTH ) )
	{
		float4& d1 = W->jdef1[j];
		if ( code == F2D_JP_LENGTH )
			d1.x = fclamp_s( v, F2D_LINEAR_SLOP, F2D_HUGE );
		else
		{
			float lo = fclamp_s( v, F2D_LINEAR_SLOP, F2D_HUGE ), hi = fclamp_s( v2, F2D_LINEAR_SLOP, F2D_HUGE );
			d1.y = fmin_s( lo, hi );
			d1.z = fmax_s( lo, hi );
		}
		clear_joint_impulses( W, j, 7 ); // impulse, lower, upper
		mark_joint_dirty( W, j );
		return;
	}
	if ( type == F2D_JOINT_MOTOR && code == F2D_JP_LINEAR_OFFSET_X )
	{
		W->jdef1[j].x = v;
		W->jdef1[j].y = v2;
		mark_joint_dirty( W, j );
		return;
	}
	if ( code == F2D_JP_UPPER || code == F2D_JP_MAX_LENGTH || code == F2D_JP_LINEAR_OFFSET_Y || code == F2D_JP_TYPE ||
		 code == F2D_JP_CURRENT || code == F2D_JP_SPEED || code == F2D_JP_MOTOR_EFFORT || code == F2D_JP_TARGET_X ||
		 code == F2D_JP_TARGET_Y || ( code >= F2D_JP_LOCAL_ANCHOR_AX && code <= F2D_JP_LOCAL_ANCHOR_BY ) )
		return; // read-only, or set through another code or call
	float* f = joint_field( W, j, type, code );
	if ( f == nullptr )
		return;
	if ( type == F2D_JOINT_MOTOR && ( code == F2D_JP_MAX_FORCE || code == F2D_JP_MAX_TORQUE ) )
		v = fmax_s( 0.0f, v );
	else if ( type == F2D_JOINT_MOTOR && code == F2D_JP_CORRECTION )
		v = fclamp_s( v, 0.0f, 1.0f );
	*f = v;
	mark_joint_dirty( W, j );
}

extern "C" F2D_API int32_t f2d_joint_get_body( int32_t index1, int32_t wg, int32_t edge, int32_t* bodyIndex1,
											   int32_t* bodyWg )
{
	*bodyIndex1 = *bodyWg = 0;
	HostWorld* W = world_from_wg( wg );
	int j = index1 - 1;
	if ( W == nullptr || j < 0 || j >= W->jointCount || !joint_live( W, j, wg ) )
		return 0;
	int b = edge == 0 ? W->jbody[j].x : W->jbody[j].y;
	*bodyIndex1 = b + 1;
	*bodyWg = pack_wg( W, W->bgen[b] );
	return 1;
}

extern "C" F2D_API void f2d_joint_wake_bodies( int32_t index1, int32_t wg )
{
	HostWorld* W = world_from_wg( wg );
	int j = index1 - 1;
	if ( W == nullptr || j < 0 || j >= W->jointCount || !joint_live( W, j, wg ) )
		return;
	for ( int e = 0; e < 2; ++e )
	{
		int b = e == 0 ? W->jbody[j].x : W->jbody[j].y;
		f2d_body_set_awake( b + 1, pack_wg( W, W->bgen[b] ), 1 );
	}
}

// ---------------------------------------------------------------------------
// step
// ---------------------------------------------------------------------------
// ---------------------------------------------------------------------------
// user callbacks, run on the host between launches (the stream is drained
// first); the device lists candidates in cbList, the host answers with the
// sorted rejected keys in cbReject
// ---------------------------------------------------------------------------
static void cb_ensure( HostWorld* W )
{
	DWorld& d = W->d;
	int cap = std::max( 1 << 16, d.contactCap );
	if ( cap <= d.cbCap )
		return;
	dgrow( d.cbList, 0, cap );
	dgrow( d.cbReject, 0, cap );
	dgrow( d.cbManifold, 0, 22 * (size_t)cap );
	d.cbCap = cap;
	W->graphDirty = true;
}

static void upload_rejected( HostWorld* W, std::vector<unsigned long long>& rejected )
{
	std::sort( rejected.begin(), rejected.end() );
	int n = (int)rejected.size();
	if ( n > 0 )
		cudaMemcpy( W->d.cbReject, rejected.data(), sizeof( unsigned long long ) * n, cudaMemcpyHostToDevice );
	cudaMemcpy( &W->d.sc->cbReject, &n, sizeof( int ), cudaMemcpyHostToDevice );
}

static int listed_count( HostWorld* W )
{
	cudaStreamSynchronize( W->stream );
	int n = 0;
	cudaMemcpy( &n, &W->d.sc->cbList, sizeof( int ), cudaMemcpyDeviceToHost );
	return std::min( n, W->d.cbCap );
}

// broad_phase.c:267-278: new pairs (sorted keys) the filter rejects are
// dropped before the contacts are created; A has the smaller proxy key
static void pair_filter_hook( void* context )
{
	HostWorld* W = (HostWorld*)context;
	DWorld& d = W->d;
	cudaStreamSynchronize( W->stream );
	int n = 0;
	cudaMemcpy( &n, &d.sc->newPairCount, sizeof( int ), cudaMemcpyDeviceToHost );
	n = std::min( n, d.pairCap );
	if ( n <= 0 )
		return;
	// the sorted pairs, decoded: (creating proxy's shape, other shape)
	std::vector<int> s1( (size_t)n ), s2( (size_t)n );
	cudaMemcpy( s1.data(), d.pairVal, sizeof( int ) * n, cudaMemcpyDeviceToHost );
	cudaMemcpy( s2.data(), d.pairValAlt, sizeof( int ) * n, cudaMemcpyDeviceToHost );
	int kept = 0;
	for ( int i = 0; i < n; ++i )
	{
		int a = s1[i], b = s2[i];
		if ( W->proxyKey[b] < W->proxyKey[a] )
			std::swap( a, b );
		if ( W->customFilter( a + 1, pack_wg( W, W->sgen[a] ), b + 1, pack_wg( W, W->sgen[b] ),
							  W->customFilterContext ) )
		{
			s1[kept] = s1[i];
			s2[kept] = s2[i];
			kept += 1;
		}
	}
	if ( kept == n )
		return;
	if ( kept > 0 )
	{
		cudaMemcpy( d.pairVal, s1.data(), sizeof( int ) * kept, cudaMemcpyHostToDevice );
		cudaMemcpy( d.pairValAlt, s2.data(), sizeof( int ) * kept, cudaMemcpyHostToDevice );
	}
	cudaMemcpy( &d.sc->newPairCount, &kept, sizeof( int ), cudaMemcpyHostToDevice );
}

// solver.c:270-280: continuous candidates (static shape, fast shape)
static void ccd_filter_hook( void* context )
{
	HostWorld* W = (HostWorld*)context;
	int n = listed_count( W );
	std::vector<unsigned long long> keys( (size_t)n ), rejected;
	if ( n > 0 )
		cudaMemcpy( keys.data(), W->d.cbList, sizeof( unsigned long long ) * n, cudaMemcpyDeviceToHost );
	for ( unsigned long long k : keys )
	{
		int ss = (int)( k >> 32 ), fs = (int)( k & 0xffffffffull );
		if ( !W->customFilter( ss + 1, pack_wg( W, W->sgen[ss] ), fs + 1, pack_wg( W, W->sgen[fs] ),
							   W->customFilterContext ) )
			rejected.push_back( k );
	}
	upload_rejected( W, rejected );
}

// contact.c:504-517: listed touching contacts with their new manifolds
static void pre_solve_hook( void* context )
{
	HostWorld* W = (HostWorld*)context;
	int n = listed_count( W );
	std::vector<unsigned long long> ids( (size_t)n ), rejected;
	std::vector<float> rec( 22 * (size_t)n );
	if ( n > 0 )
	{
		cudaMemcpy( ids.data(), W->d.cbList, sizeof( unsigned long long ) * n, cudaMemcpyDeviceToHost );
		cudaMemcpy( rec.data(), W->d.cbManifold, sizeof( float ) * 22 * n, cudaMemcpyDeviceToHost );
	}
	for ( int i = 0; i < n; ++i )
	{
		const float* r = rec.data() + 22 * (size_t)i;
		f2d_manifold_view v;
		static_assert( sizeof( f2d_manifold_view ) == 20 * sizeof( float ), "manifold view layout" );
		memcpy( &v, r, sizeof( v ) );
		int a = float_to_bits( r[20] ), b = float_to_bits( r[21] );
		if ( !W->preSolve( a + 1, pack_wg( W, W->sgen[a] ), b + 1, pack_wg( W, W->sgen[b] ), &v, W->preSolveContext ) )
			rejected.push_back( ids[i] );
	}
	upload_rejected( W, rejected );
}

extern "C" F2D_API void f2d_world_set_custom_filter( int32_t worldId, f2d_custom_filter_fn fn, void* context )
{
	HostWorld* W = world_from_id( worldId );
	if ( W == nullptr )
		return;
	W->customFilter = fn;
	W->customFilterContext = context;
	W->d.callbacks = ( W->d.callbacks & ~1 ) | ( fn ? 1 : 0 );
	W->graphDirty = true;
}

extern "C" F2D_API void f2d_world_set_pre_solve( int32_t worldId, f2d_pre_solve_fn fn, void* context )
{
	HostWorld* W = world_from_id( worldId );
	if ( W == nullptr )
		return;
	W->preSolve = fn;
	W->preSolveContext = context;
	W->d.callbacks = ( W->d.callbacks & ~2 ) | ( fn ? 2 : 0 );
	W->graphDirty = true;
}

static void enqueue_step( HostWorld* W, float dt, int subSteps, int planMode )
{
	DWorld& d = W->d;
	bool prof = W->profiling;
	if ( prof && W->ph[0] == nullptr )
		for ( int i = 0; i < 9; ++i )
			cudaEventCreate( W->ph + i );
	W->s.evSolveStart = prof ? W->ph[4] : nullptr;
	launch_reset_counters( d, W->stream );
	if ( prof )
		cudaEventRecord( W->ph[0], W->stream );
	bool filter = W->customFilter != nullptr, pre = W->preSolve != nullptr;
	W->s.rebuildT0 = prof ? W->ph[7] : nullptr;
	W->s.rebuildT1 = prof ? W->ph[8] : nullptr;
	// the tree rebuild forks onto its own stream inside the broadphase
	launch_broadphase( d, W->s, W->stream, planMode, filter ? pair_filter_hook : nullptr, W );
	if ( prof )
		cudaEventRecord( W->ph[1], W->stream );
	launch_narrowphase( d, W->s, W->stream, pre ? pre_solve_hook : nullptr, W );
	if ( prof )
		cudaEventRecord( W->ph[2], W->stream );
	launch_graph( d, W->s, W->stream );
	cudaStreamWaitEvent( W->stream, W->s.rebuildJoin, 0 );
	if ( prof )
		cudaEventRecord( W->ph[3], W->stream );
	launch_solver( d, W->s, W->stream, dt, subSteps );
	if ( d.learnMode & 1 )
		launch_record_samples( d, W->stream );
	if ( prof )
		cudaEventRecord( W->ph[5], W->stream );
	launch_finalize( d, W->s, W->stream, dt, filter ? ccd_filter_hook : nullptr, W );
	launch_sensors( d, W->s, W->stream );
	if ( prof )
		cudaEventRecord( W->ph[6], W->stream );
	W->s.evSolveStart = nullptr;
}

static int count_kernel_nodes( cudaGraph_t g )
{
	size_t n = 0;
	cudaGraphGetNodes( g, nullptr, &n );
	std::vector<cudaGraphNode_t> nodes( n );
	cudaGraphGetNodes( g, nodes.data(), &n );
	int k = 0;
	for ( size_t i = 0; i < n; ++i )
	{
		cudaGraphNodeType t;
		cudaGraphNodeGetType( nodes[i], &t );
		if ( t == cudaGraphNodeTypeKernel )
			k += 1;
	}
	return k;
}

static void ensure_learning_buffers( HostWorld* W );

extern "C" F2D_API int32_t f2d_world_step( int32_t worldId, double timeStep, int32_t subStepCount )
{
	HostWorld* W = world_from_id( worldId );
	if ( W == nullptr )
		return F2D_STATUS_INVALID;
	float dt = (float)timeStep;
	// world.c:717-725, :808-810: the end events of destroys since the last
	// step are reported with this one; a zero step reports only those
	W->endPrefix.swap( W->endNext );
	W->endNext.clear();
	W->sensorEndPrefix.swap( W->sensorEndNext );
	W->sensorEndNext.clear();
	if ( dt == 0.0f )
	{
		W->eventsCleared = true;
		return 0;
	}
	W->eventsCleared = false;
	int subSteps = subStepCount < 1 ? 1 : subStepCount;
	float inv_dt = 1.0f / dt;
	W->invH = (float)subSteps * inv_dt;
	// collect the status of earlier steps without blocking
	if ( W->stepped && cudaEventQuery( W->evStop ) == cudaSuccess )
		W->statusAccum |= *W->hostError;
	flush_uploads( W );
	upload_host_moves( W );
	int planMode = 0;
	if ( W->planPending )
	{
		int n = (int)W->planKeys.size();
		if ( n > W->d.pairCap )
			n = W->d.pairCap;
		cudaMemcpyAsync( W->d.planKeys, W->planKeys.data(), sizeof( unsigned long long ) * n, cudaMemcpyHostToDevice,
						 W->stream );
		cudaMemcpyAsync( W->d.planIds, W->planIds.data(), sizeof( int ) * n, cudaMemcpyHostToDevice, W->stream );
		cudaMemcpyAsync( &W->d.sc->planCount, &n, sizeof( int ), cudaMemcpyHostToDevice, W->stream );
		cudaStreamSynchronize( W->stream );
		W->planPending = false;
		planMode = 1;
	}
	if ( W->d.learnMode != 0 )
		ensure_learning_buffers( W );
	cudaMemsetAsync( &W->d.sc->error, 0, sizeof( int ), W->stream );
	if ( W->forceRebuild )
	{
		cudaMemsetAsync( &W->d.sc->forceRebuild, 1, 1, W->stream );
		W->forceRebuild = false;
	}
	cudaEventRecord( W->evStart, W->stream );
	if ( W->d.callbacks )
		cb_ensure( W );
	bool useGraph = planMode == 0 && !W->profiling && W->d.callbacks == 0;
	if ( useGraph && ( W->graphDirty || W->graphExec == nullptr || W->graphDt != dt || W->graphSubSteps != subSteps ) )
	{
		if ( W->graphExec )
		{
			cudaGraphExecDestroy( W->graphExec );
			W->graphExec = nullptr;
		}
		cudaGraph_t g;
		if ( cudaStreamBeginCapture( W->stream, cudaStreamCaptureModeThreadLocal ) == cudaSuccess )
		{
			enqueue_step( W, dt, subSteps, 0 );
			if ( cudaStreamEndCapture( W->stream, &g ) == cudaSuccess )
			{
				if ( cudaGraphInstantiate( &W->graphExec, g, 0 ) != cudaSuccess )
					W->graphExec = nullptr;
				W->graphKernelNodes = count_kernel_nodes( g );
				cudaGraphDestroy( g );
			}
		}
		cudaGetLastError();
		W->graphDt = dt;
		W->graphSubSteps = subSteps;
		W->graphDirty = false;
	}
	if ( useGraph && W->graphExec )
	{
		cudaGraphLaunch( W->graphExec, W->stream );
		W->lastLaunches = W->graphKernelNodes;
	}
	else
	{
		enqueue_step( W, dt, subSteps, planMode );
		W->lastLaunches = W->graphKernelNodes;
	}
	cudaEventRecord( W->evStop, W->stream );
	cudaMemcpyAsync( W->hostError, &W->d.sc->error, sizeof( int ), cudaMemcpyDeviceToHost, W->stream );
	W->stepped = true;
	// the step enlarged and rebuilt the kinematic and dynamic trees and
	// changed every awake body row
	W->treeStale[1] = true;
	W->treeStale[2] = true;
	body_rows_changed( W, true );
	cudaError_t e = cudaGetLastError();
	if ( e != cudaSuccess )
		W->statusAccum |= F2D_STATUS_CUDA;
	int st = W->statusAccum;
	W->statusAccum = 0;
	return st;
}

// ---------------------------------------------------------------------------
// autotuner: launch shapes that change timing but never results
// ---------------------------------------------------------------------------
static void apply_tuning( HostWorld* W, int variant, int period )
{
	W->s.solverVariant = variant;
	W->orderPeriod = period;
	cudaMemcpyAsync( &W->d.sc->orderPeriod, &W->orderPeriod, sizeof( int ), cudaMemcpyHostToDevice, W->stream );
	cudaStreamSynchronize( W->stream );
	W->graphDirty = true;
}

extern "C" F2D_API int32_t f2d_world_autotune( int32_t worldId, double timeStep, int32_t subStepCount,
											   int32_t stepsPerCandidate, int32_t* chosen3 )
{
	HostWorld* W = world_from_id( worldId );
	if ( W == nullptr )
		return F2D_STATUS_INVALID;
	flush_uploads( W );
	int variants[3];
	int nv = 0;
	if ( W->s.clusterCapacity > 0 && W->bodyCount <= W->s.clusterCapacity )
		variants[nv++] = SOLVER_CLUSTER;
	variants[nv++] = SOLVER_GRID512;
	if ( W->s.solverBlocks256 > 0 )
		variants[nv++] = SOLVER_GRID256;
	const int periods[4] = { 4, 8, 16, 32 };
	int reps = stepsPerCandidate < 1 ? 1 : stepsPerCandidate;
	int status = 0;
	int taken = 0;
	double best = 1e30;
	int bestV = SOLVER_AUTO, bestP = 0;
	for ( int vi = 0; vi < nv; ++vi )
		for ( int pi = 0; pi < 4; ++pi )
		{
			apply_tuning( W, variants[vi], periods[pi] );
			// the first step re-captures the graph; the leaf order is re-sorted
			// at least once per period, so a candidate is timed over a period
			status |= f2d_world_step( worldId, timeStep, subStepCount );
			int n = reps > periods[pi] ? reps : periods[pi];
			taken += 1 + n;
			double ms = 0.0;
			for ( int k = 0; k < n; ++k )
			{
				status |= f2d_world_step( worldId, timeStep, subStepCount );
				ms += f2d_world_last_step_ms( worldId );
			}
			ms /= n;
			if ( ms < best )
			{
				best = ms;
				bestV = variants[vi];
				bestP = periods[pi];
			}
		}
	apply_tuning( W, bestV, bestP );
	if ( chosen3 )
	{
		chosen3[0] = bestV;
		chosen3[1] = bestP;
		chosen3[2] = taken;
	}
	return status | f2d_world_sync( worldId );
}

extern "C" F2D_API void f2d_world_get_tuning( int32_t worldId, int32_t* out2 )
{
	HostWorld* W = world_from_id( worldId );
	out2[0] = W ? W->s.solverVariant : 0;
	out2[1] = W ? W->orderPeriod : 0;
}

// ---------------------------------------------------------------------------
// learned warm start: sample recording and model binding
// ---------------------------------------------------------------------------
bool f2d_internal_mlp_valid( int32_t handle ); // mlp.cu

static void ensure_learning_buffers( HostWorld* W )
{
	DWorld& d = W->d;
	if ( d.newPointCap < d.contactCap )
	{
		cudaStreamSynchronize( W->stream );
		dfree( d.newPoint );
		dfree( d.newFeat );
		dgrow( d.newPoint, 0, (size_t)d.contactCap );
		dgrow( d.newFeat, 0, (size_t)d.contactCap * 12 );
		d.newPointCap = d.contactCap;
	}
}

extern "C" F2D_API void f2d_world_set_sample_recording( int32_t worldId, int32_t capacity )
{
	HostWorld* W = world_from_id( worldId );
	if ( W == nullptr )
		return;
	cudaStreamSynchronize( W->stream );
	DWorld& d = W->d;
	dfree( d.samples );
	d.sampleCap = 0;
	if ( capacity > 0 )
	{
		dgrow( d.samples, 0, (size_t)capacity * 14 );
		d.sampleCap = capacity;
		ensure_learning_buffers( W );
		d.learnMode |= 1;
	}
	else
		d.learnMode &= ~1;
	cudaMemsetAsync( &d.sc->sampleCount, 0, sizeof( int ), W->stream );
	W->graphDirty = true;
}

extern "C" F2D_API int32_t f2d_world_sample_count( int32_t worldId )
{
	HostWorld* W = world_from_id( worldId );
	if ( W == nullptr )
		return 0;
	cudaStreamSynchronize( W->stream );
	int n = 0;
	cudaMemcpy( &n, &W->d.sc->sampleCount, sizeof( int ), cudaMemcpyDeviceToHost );
	return std::min( n, W->d.sampleCap );
}

extern "C" F2D_API int32_t f2d_world_get_samples( int32_t worldId, float* out14, int32_t capacity )
{
	int n = std::min( f2d_world_sample_count( worldId ), capacity );
	HostWorld* W = world_from_id( worldId );
	if ( W == nullptr || n <= 0 )
		return 0;
	cudaMemcpy( out14, W->d.samples, sizeof( float ) * 14 * (size_t)n, cudaMemcpyDeviceToHost );
	return n;
}

extern "C" F2D_API int32_t f2d_world_set_warm_start_model( int32_t worldId, int32_t model )
{
	HostWorld* W = world_from_id( worldId );
	if ( W == nullptr )
		return 0;
	cudaStreamSynchronize( W->stream );
	if ( model > 0 && f2d_internal_mlp_valid( model ) )
	{
		ensure_learning_buffers( W );
		W->d.mlpModel = model - 1;
		W->d.learnMode |= 2;
	}
	else
	{
		W->d.mlpModel = -1;
		W->d.learnMode &= ~2;
	}
	W->graphDirty = true;
	return 1;
}

extern "C" F2D_API int32_t f2d_world_sync( int32_t worldId )
{
	HostWorld* W = world_from_id( worldId );
	if ( W == nullptr )
		return F2D_STATUS_INVALID;
	cudaError_t e = cudaStreamSynchronize( W->stream );
	int st = W->statusAccum | ( W->stepped ? *W->hostError : 0 );
	if ( e != cudaSuccess )
		st |= F2D_STATUS_CUDA;
	if ( W->stepped )
	{
		float ms = 0.0f;
		cudaEventElapsedTime( &ms, W->evStart, W->evStop );
		W->lastStepMs = ms;
	}
	W->statusAccum = 0;
	*W->hostError = 0;
	return st;
}

extern "C" F2D_API double f2d_world_last_step_ms( int32_t worldId )
{
	HostWorld* W = world_from_id( worldId );
	if ( W == nullptr || !W->stepped )
		return 0.0;
	cudaEventSynchronize( W->evStop );
	float ms = 0.0f;
	cudaEventElapsedTime( &ms, W->evStart, W->evStop );
	return ms;
}

extern "C" F2D_API int32_t f2d_world_last_step_launches( int32_t worldId )
{
	HostWorld* W = world_from_id( worldId );
	return W ? W->lastLaunches : 0;
}

extern "C" F2D_API void f2d_world_set_contact_plan( int32_t worldId, const int32_t* rows, int32_t count )
{
	HostWorld* W = world_from_id( worldId );
	if ( W == nullptr )
		return;
	std::vector<std::pair<unsigned long long, int>> v;
	for ( int i = 0; i < count; ++i )
	{
		int id = rows[3 * i], a = rows[3 * i + 1], b = rows[3 * i + 2];
		unsigned long long key = a < b ? ( ( (unsigned long long)a << 32 ) | (unsigned)b )
									   : ( ( (unsigned long long)b << 32 ) | (unsigned)a );
		v.push_back( std::make_pair( key, id ) );
	}
	std::sort( v.begin(), v.end() );
	W->planKeys.resize( v.size() );
	W->planIds.resize( v.size() );
	for ( size_t i = 0; i < v.size(); ++i )
	{
		W->planKeys[i] = v[i].first;
		W->planIds[i] = v[i].second;
	}
	W->planPending = true;
}

// ---------------------------------------------------------------------------
// world settings
// ---------------------------------------------------------------------------
extern "C" F2D_API void f2d_world_set_gravity( int32_t worldId, double x, double y )
{
	HostWorld* W = world_from_id( worldId );
	if ( W == nullptr )
		return;
	W->d.gravity = mk( (float)x, (float)y );
	W->graphDirty = true;
}

extern "C" F2D_API int32_t f2d_world_begin_subworld( int32_t worldId, double gravityX, double gravityY )
{
	HostWorld* W = world_from_id( worldId );
	if ( W == nullptr )
		return -1;
	W->subGravity = make_float2( (float)gravityX, (float)gravityY );
	W->d.subCount += 1;
	W->graphDirty = true;
	return W->d.subCount - 1;
}

extern "C" F2D_API int32_t f2d_world_subworld_count( int32_t worldId )
{
	HostWorld* W = world_from_id( worldId );
	return W ? W->d.subCount : 0;
}

extern "C" F2D_API void f2d_world_get_gravity( int32_t worldId, double* x, double* y )
{
	HostWorld* W = world_from_id( worldId );
	if ( W == nullptr )
		return;
	*x = W->d.gravity.x;
	*y = W->d.gravity.y;
}

extern "C" F2D_API void f2d_world_enable_sleeping( int32_t worldId, int32_t enabled )
{
	HostWorld* W = world_from_id( worldId );
	if ( W == nullptr )
		return;
	if ( ( enabled != 0 ) == ( W->d.enableSleep != 0 ) )
		return;
	W->d.enableSleep = enabled != 0;
	W->graphDirty = true;
	// world.c:1726-1738: disabling wakes every sleeping set
	if ( !enabled && W->islOn && W->d.isl )
	{
		flush_uploads( W );
		launch_isl_api( W->d, W->stream, 2, 0 );
		body_rows_changed( W, false );
	}
}

extern "C" F2D_API int32_t f2d_world_is_sleeping_enabled( int32_t worldId )
{
	HostWorld* W = world_from_id( worldId );
	return W ? W->d.enableSleep : 0;
}

extern "C" F2D_API void f2d_world_enable_continuous( int32_t worldId, int32_t enabled )
{
	HostWorld* W = world_from_id( worldId );
	if ( W == nullptr )
		return;
	W->d.enableContinuous = enabled != 0;
	W->graphDirty = true;
}

extern "C" F2D_API int32_t f2d_world_is_continuous_enabled( int32_t worldId )
{
	HostWorld* W = world_from_id( worldId );
	return W ? W->d.enableContinuous : 0;
}

// ---------------------------------------------------------------------------
// body accessors
// ---------------------------------------------------------------------------
extern "C" F2D_API int32_t f2d_body_is_valid( int32_t index1, int32_t wg )
{
	HostWorld* W;
	return body_from( index1, wg, &W ) >= 0;
}

extern "C" F2D_API void f2d_body_get_position( int32_t index1, int32_t wg, double* x, double* y )
{
	HostWorld* W;
	int b = body_from( index1, wg, &W );
	if ( b < 0 )
		return;
	pull_body( W, b );
	*x = W->xf[b].x;
	*y = W->xf[b].y;
}

extern "C" F2D_API void f2d_body_get_rotation( int32_t index1, int32_t wg, double* c, double* s )
{
	HostWorld* W;
	int b = body_from( index1, wg, &W );
	if ( b < 0 )
		return;
	pull_body( W, b );
	*c = W->xf[b].z;
	*s = W->xf[b].w;
}

extern "C" F2D_API void f2d_body_set_transform( int32_t index1, int32_t wg, double px, double py, double c, double s )
{
	HostWorld* W;
	int b = body_from( index1, wg, &W );
	if ( b < 0 )
		return;
	pull_body( W, b );
	frot q;
	q.c = (float)c;
	q.s = (float)s;
	fv2 p = mk( (float)px, (float)py );
	W->xf[b] = make_float4( p.x, p.y, q.c, q.s );
	float2 lc = W->localCenter[b];
	fv2 cc = vadd( rrot( q, mk( lc.x, lc.y ) ), p );
	W->center[b] = make_float2( cc.x, cc.y );
	W->sweep0[b] = make_float4( cc.x, cc.y, q.c, q.s );
	// refresh shape boxes and re-enter the move buffer (body.c:720-780)
	fxf xf;
	xf.p = p;
	xf.q = q;
	int proxyType = body_type( W->bflags[b] );
	for ( int sh = W->headShape[b]; sh != F2D_NULL; sh = W->nextShape[sh] )
	{
		if ( sh < W->shapeUploaded )
		{
			cudaStreamSynchronize( W->stream );
			down( W->sflags, W->d.sflags, sh, sh + 1 );
		}
		fbox aabb = box_grow( h_shape_aabb( W->hgeomv[sh], xf ), F2D_SPECULATIVE );
		float margin = proxyType == 0 ? F2D_SPECULATIVE : F2D_AABB_MARGIN;
		W->aabb[sh] = box_to4( aabb );
		W->fat[sh] = box_to4( box_grow( aabb, margin ) );
		// broad_phase.c:116-123 b2BroadPhase_MoveProxy: re-insert, then buffer
		int pk = W->proxyKey[sh];
		if ( pk != F2D_NULL )
		{
			tree_pull( W, pk & 3 );
			W->trees[pk & 3].move_proxy( pk >> 2, W->fat[sh] );
			W->treeDirty[pk & 3] = true;
			host_move( W, sh );
			if ( ( pk & 3 ) == 0 )
				W->staticDirty = true;
		}
		mark_shape( W, sh );
	}
	mark_body( W, b );
}

extern "C" F2D_API void f2d_body_get_linear_velocity( int32_t index1, int32_t wg, double* x, double* y )
{
	HostWorld* W;
	int b = body_from( index1, wg, &W );
	if ( b < 0 )
		return;
	pull_body( W, b );
	*x = W->vel[b].x;
	*y = W->vel[b].y;
}

// Sleeping worlds: the wake of an edit (body.c b2WakeBody) runs on the device
// before the row is read back; an edit of a body that stays asleep is
// dropped, as the reference finds no body state for it. Returns whether the
// edit applies.
static int isl_set_of( HostWorld* W, int b )
{
	int s = SET_AWAKE;
	cudaStreamSynchronize( W->stream );
	cudaMemcpy( &s, W->islHost.bSet + b, sizeof( int ), cudaMemcpyDeviceToHost );
	return s;
}

static bool isl_edit( HostWorld* W, int b, bool wake )
{
	if ( !W->islOn )
		return true;
	flush_uploads( W );
	if ( wake )
	{
		launch_isl_api( W->d, W->stream, 0, b );
		body_rows_changed( W, false );
	}
	return isl_set_of( W, b ) == SET_AWAKE;
}

extern "C" F2D_API void f2d_body_set_linear_velocity( int32_t index1, int32_t wg, double x, double y )
{
	HostWorld* W;
	int b = body_from( index1, wg, &W );
	if ( b < 0 || body_type( W->bflags[b] ) == 0 )
		return;
	if ( !isl_edit( W, b, (float)x * (float)x + (float)y * (float)y > 0.0f ) )
		return;
	pull_body( W, b );
	W->vel[b].x = (float)x;
	W->vel[b].y = (float)y;
	mark_body( W, b );
}

extern "C" F2D_API double f2d_body_get_angular_velocity( int32_t index1, int32_t wg )
{
	HostWorld* W;
	int b = body_from( index1, wg, &W );
	if ( b < 0 )
		return 0.0;
	pull_body( W, b );
	return W->vel[b].z;
}

extern "C" F2D_API void f2d_body_set_angular_velocity( int32_t index1, int32_t wg, double w )
{
	HostWorld* W;
	int b = body_from( index1, wg, &W );
	if ( b < 0 || body_type( W->bflags[b] ) == 0 )
		return;
	if ( !isl_edit( W, b, (float)w != 0.0f ) )
		return;
	pull_body( W, b );
	W->vel[b].z = (float)w;
	mark_body( W, b );
}

// body.c:1000-1110 (b2Body_ApplyForce ... ApplyAngularImpulse)
extern "C" F2D_API void f2d_body_apply_force( int32_t index1, int32_t wg, double fx, double fy, double px, double py,
											  int32_t wake )
{
	HostWorld* W;
	int b = body_from( index1, wg, &W );
	if ( b < 0 || body_type( W->bflags[b] ) != 2 )
		return;
	if ( !isl_edit( W, b, wake != 0 ) )
		return;
	pull_body( W, b );
	fv2 f = mk( (float)fx, (float)fy );
	fv2 c = mk( W->center[b].x, W->center[b].y );
	float4 fo = W->force[b];
	fo.x += f.x;
	fo.y += f.y;
	fo.z += vcross( vsub( mk( (float)px, (float)py ), c ), f );
	W->force[b] = fo;
	mark_body( W, b );
}

extern "C" F2D_API void f2d_body_apply_force_to_center( int32_t index1, int32_t wg, double fx, double fy, int32_t wake )
{
	HostWorld* W;
	int b = body_from( index1, wg, &W );
	if ( b < 0 || body_type( W->bflags[b] ) != 2 )
		return;
	if ( !isl_edit( W, b, wake != 0 ) )
		return;
	pull_body( W, b );
	W->force[b].x += (float)fx;
	W->force[b].y += (float)fy;
	mark_body( W, b );
}

extern "C" F2D_API void f2d_body_apply_torque( int32_t index1, int32_t wg, double torque, int32_t wake )
{
	HostWorld* W;
	int b = body_from( index1, wg, &W );
	if ( b < 0 || body_type( W->bflags[b] ) != 2 )
		return;
	if ( !isl_edit( W, b, wake != 0 ) )
		return;
	pull_body( W, b );
	W->force[b].z += (float)torque;
	mark_body( W, b );
}

extern "C" F2D_API void f2d_body_apply_linear_impulse( int32_t index1, int32_t wg, double ix, double iy, double px,
													   double py, int32_t wake )
{
	HostWorld* W;
	int b = body_from( index1, wg, &W );
	if ( b < 0 || body_type( W->bflags[b] ) != 2 )
		return;
	if ( !isl_edit( W, b, wake != 0 ) )
		return;
	pull_body( W, b );
	fv2 impulse = mk( (float)ix, (float)iy );
	fv2 c = mk( W->center[b].x, W->center[b].y );
	float4 v = W->vel[b];
	float invMass = W->massv[b].x, invI = W->massv[b].y;
	fv2 nv = vmuladd( mk( v.x, v.y ), invMass, impulse );
	float nw = v.z + invI * vcross( vsub( mk( (float)px, (float)py ), c ), impulse );
	W->vel[b] = make_float4( nv.x, nv.y, nw, v.w );
	mark_body( W, b );
}

extern "C" F2D_API void f2d_body_apply_linear_impulse_to_center( int32_t index1, int32_t wg, double ix, double iy,
																 int32_t wake )
{
	HostWorld* W;
	int b = body_from( index1, wg, &W );
	if ( b < 0 || body_type( W->bflags[b] ) != 2 )
		return;
	if ( !isl_edit( W, b, wake != 0 ) )
		return;
	pull_body( W, b );
	float4 v = W->vel[b];
	float invMass = W->massv[b].x;
	fv2 nv = vmuladd( mk( v.x, v.y ), invMass, mk( (float)ix, (float)iy ) );
	W->vel[b] = make_float4( nv.x, nv.y, v.z, v.w );
	mark_body( W, b );
}

extern "C" F2D_API void f2d_body_apply_angular_impulse( int32_t index1, int32_t wg, double impulse, int32_t wake )
{
	HostWorld* W;
	int b = body_from( index1, wg, &W );
	if ( b < 0 || body_type( W->bflags[b] ) != 2 )
		return;
	if ( !isl_edit( W, b, wake != 0 ) )
		return;
	pull_body( W, b );
	W->vel[b].z += W->massv[b].y * (float)impulse;
	mark_body( W, b );
}

extern "C" F2D_API double f2d_body_get_mass( int32_t index1, int32_t wg )
{
	HostWorld* W;
	int b = body_from( index1, wg, &W );
	return b < 0 ? 0.0 : W->bmass[b];
}

extern "C" F2D_API double f2d_body_get_rotational_inertia( int32_t index1, int32_t wg )
{
	HostWorld* W;
	int b = body_from( index1, wg, &W );
	return b < 0 ? 0.0 : W->binertia[b];
}

extern "C" F2D_API int32_t f2d_body_get_type( int32_t index1, int32_t wg )
{
	HostWorld* W;
	int b = body_from( index1, wg, &W );
	return b < 0 ? -1 : body_type( W->bflags[b] );
}

extern "C" F2D_API int32_t f2d_body_is_awake( int32_t index1, int32_t wg )
{
	HostWorld* W;
	int b = body_from( index1, wg, &W );
	if ( b < 0 )
		return 0;
	if ( W->islOn )
	{
		flush_uploads( W );
		return isl_set_of( W, b ) == SET_AWAKE;
	}
	return body_type( W->bflags[b] ) != 0 && ( W->bflags[b] & BF_ENABLED );
}

// RawBox2D.bodySetAwake (raw_box2d.dart:232 -> b2Body_SetAwake, body.c:1483-1508)
extern "C" F2D_API void f2d_body_set_awake( int32_t index1, int32_t wg, int32_t awake )
{
	HostWorld* W;
	int b = body_from( index1, wg, &W );
	if ( b < 0 || !W->islOn )
		return;
	flush_uploads( W );
	launch_isl_api( W->d, W->stream, awake ? 0 : 1, b );
	body_rows_changed( W, false );
}

// RawBox2D.worldExplode (raw_box2d.dart:1342 -> b2World_Explode, world.c:2718):
// enqueued on the world's stream after the pending uploads
extern "C" F2D_API void f2d_world_explode( int32_t worldId, int64_t maskBits, double positionX, double positionY,
										   double radius, double falloff, double impulsePerLength )
{
	HostWorld* W = world_from_id( worldId );
	if ( W == nullptr || W->shapeCount == 0 )
		return;
	flush_uploads( W );
	launch_explode( W->d, W->stream, W->s.tmpA, (unsigned long long)maskBits, (float)positionX, (float)positionY,
					(float)radius, (float)falloff, (float)impulsePerLength );
	body_rows_changed( W, true );
}

// RawBox2D.bodyIsSleepEnabled / bodyEnableSleep (raw_box2d.dart:235-242;
// b2Body_EnableSleep wakes the body when sleep is disabled)
extern "C" F2D_API int32_t f2d_body_is_sleep_enabled( int32_t index1, int32_t wg )
{
	HostWorld* W;
	int b = body_from( index1, wg, &W );
	return b < 0 ? 0 : ( W->bflags[b] & BF_ENABLE_SLEEP ) != 0;
}

extern "C" F2D_API void f2d_body_enable_sleep( int32_t index1, int32_t wg, int32_t enabled )
{
	HostWorld* W;
	int b = body_from( index1, wg, &W );
	if ( b < 0 )
		return;
	if ( !enabled && W->islOn )
	{
		flush_uploads( W );
		launch_isl_api( W->d, W->stream, 0, b );
		body_rows_changed( W, false );
	}
	pull_body( W, b );
	if ( enabled )
		W->bflags[b] |= BF_ENABLE_SLEEP;
	else
		W->bflags[b] &= ~BF_ENABLE_SLEEP;
	mark_body( W, b );
}

// RawBox2D.bodyGetSleepThreshold / bodySetSleepThreshold (raw_box2d.dart:245-248)
extern "C" F2D_API double f2d_body_get_sleep_threshold( int32_t index1, int32_t wg )
{
	HostWorld* W;
	int b = body_from( index1, wg, &W );
	return b < 0 ? 0.0 : W->damp[b].w;
}

extern "C" F2D_API void f2d_body_set_sleep_threshold( int32_t index1, int32_t wg, double value )
{
	HostWorld* W;
	int b = body_from( index1, wg, &W );
	if ( b < 0 )
		return;
	pull_body( W, b );
	W->damp[b].w = (float)value;
	mark_body( W, b );
}

// ---------------------------------------------------------------------------
// bulk readers
// ---------------------------------------------------------------------------
extern "C" F2D_API int32_t f2d_world_body_capacity( int32_t worldId )
{
	HostWorld* W = world_from_id( worldId );
	return W ? W->bodyCount : 0;
}

// Packs the bulk body rows on the device so that one copy brings them home.
__global__ void k_pack_bodies( DWorld w, float* out, int n )
{
	for ( int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x )
	{
		float* o = out + 12 * (size_t)i;
		int f = w.bflags[i];
		if ( ( f & BF_USED ) == 0 )
		{
			for ( int k = 0; k < 12; ++k )
				o[k] = 0.0f;
			continue;
		}
		float4 x = w.xf[i], v = w.vel[i], fo = w.force[i];
		float2 c = w.center[i];
		o[0] = x.x;
		o[1] = x.y;
		o[2] = x.z;
		o[3] = x.w;
		o[4] = v.x;
		o[5] = v.y;
		o[6] = v.z;
		o[7] = c.x;
		o[8] = c.y;
		o[9] = 1.0f;
		o[10] = w.isl ? (float)w.isl->bSet[i] : ( body_type( f ) == 0 ? 0.0f : 2.0f );
		o[11] = fo.w;
	}
}

static void host_body_row( const HostWorld* W, int i, float* o )
{
	memset( o, 0, sizeof( float ) * 12 );
	if ( ( W->bflags[i] & BF_USED ) == 0 )
		return;
	o[0] = W->xf[i].x;
	o[1] = W->xf[i].y;
	o[2] = W->xf[i].z;
	o[3] = W->xf[i].w;
	o[4] = W->vel[i].x;
	o[5] = W->vel[i].y;
	o[6] = W->vel[i].z;
	o[7] = W->center[i].x;
	o[8] = W->center[i].y;
	o[9] = 1.0f;
	o[10] = body_type( W->bflags[i] ) == 0 ? 0.0f : 2.0f;
	o[11] = W->force[i].w;
}

extern "C" F2D_API int32_t f2d_world_get_bodies( int32_t worldId, float* out, int32_t cap )
{
	HostWorld* W = world_from_id( worldId );
	if ( W == nullptr )
		return 0;
	int n = std::min( W->bodyCount, cap );
	int up = std::min( n, W->bodyUploaded );
	if ( up > 0 )
	{
		if ( W->packedCap < W->d.bodyCap )
		{
			cudaStreamSynchronize( W->stream );
			if ( W->packedBodies )
				cudaFree( W->packedBodies );
			cudaMalloc( (void**)&W->packedBodies, sizeof( float ) * 12 * (size_t)W->d.bodyCap );
			W->packedCap = W->d.bodyCap;
		}
		k_pack_bodies<<<grid_for( up ), 256, 0, W->stream>>>( W->d, W->packedBodies, up );
		cudaMemcpyAsync( out, W->packedBodies, sizeof( float ) * 12 * (size_t)up, cudaMemcpyDeviceToHost, W->stream );
		cudaStreamSynchronize( W->stream );
		// rows edited on the host since the last upload are newer than the device
		for ( int b : W->bodyDirty )
			if ( b < up )
				host_body_row( W, b, out + 12 * (size_t)b );
	}
	for ( int i = up; i < n; ++i )
		host_body_row( W, i, out + 12 * (size_t)i );
	return n;
}

extern "C" F2D_API int32_t f2d_world_contact_capacity( int32_t worldId )
{
	HostWorld* W = world_from_id( worldId );
	if ( W == nullptr )
		return 0;
	cudaStreamSynchronize( W->stream );
	DScalars sc;
	cudaMemcpy( &sc, W->d.sc, sizeof( sc ), cudaMemcpyDeviceToHost );
	return sc.contactIdCount;
}

extern "C" F2D_API int32_t f2d_world_get_contacts( int32_t worldId, int32_t* ints, float* floats, int32_t cap )
{
	HostWorld* W = world_from_id( worldId );
	if ( W == nullptr )
		return 0;
	cudaStreamSynchronize( W->stream );
	DScalars sc;
	cudaMemcpy( &sc, W->d.sc, sizeof( sc ), cudaMemcpyDeviceToHost );
	int n = sc.contactIdCount;
	std::vector<int2> cs( n );
	std::vector<int> cf( n ), cc( n );
	std::vector<float4> mn( n ), pa( 2 * (size_t)n ), pb( 2 * (size_t)n ), pi( 2 * (size_t)n );
	if ( n > 0 )
	{
		cudaMemcpy( cs.data(), W->d.cshape, sizeof( int2 ) * n, cudaMemcpyDeviceToHost );
		cudaMemcpy( cf.data(), W->d.cflags, sizeof( int ) * n, cudaMemcpyDeviceToHost );
		cudaMemcpy( cc.data(), W->d.ccolor, sizeof( int ) * n, cudaMemcpyDeviceToHost );
		cudaMemcpy( mn.data(), W->d.mnorm, sizeof( float4 ) * n, cudaMemcpyDeviceToHost );
		cudaMemcpy( pa.data(), W->d.mpA, sizeof( float4 ) * 2 * n, cudaMemcpyDeviceToHost );
		cudaMemcpy( pb.data(), W->d.mpB, sizeof( float4 ) * 2 * n, cudaMemcpyDeviceToHost );
		cudaMemcpy( pi.data(), W->d.mpI, sizeof( float4 ) * 2 * n, cudaMemcpyDeviceToHost );
	}
	int m = 0;
	for ( int id = 0; id < n && m < cap; ++id )
	{
		if ( ( cf[id] & CF_USED ) == 0 )
			continue;
		int* oi = ints + 9 * m;
		float* of = floats + 25 * m;
		int count = float_to_bits( mn[id].w );
		oi[0] = id;
		oi[1] = cs[id].x;
		oi[2] = cs[id].y;
		oi[3] = cc[id];
		oi[4] = count;
		oi[5] = ( ( cf[id] & CF_TOUCHING ) ? 1 : 0 ) | ( ( cf[id] & CF_EVENTS ) ? 2 : 0 );
		oi[6] = cf[id] & 0xffff0000;
		oi[7] = float_to_bits( pb[2 * id].w ) & 0xffff;
		oi[8] = float_to_bits( pb[2 * id + 1].w ) & 0xffff;
		of[0] = mn[id].x;
		of[1] = mn[id].y;
		of[2] = mn[id].z;
		for ( int k = 0; k < 2; ++k )
		{
			float* p = of + 3 + 11 * k;
			float4 a = pa[2 * id + k], b = pb[2 * id + k], im = pi[2 * id + k];
			p[0] = a.x;
			p[1] = a.y;
			p[2] = a.z;
			p[3] = a.w;
			p[4] = b.x;
			p[5] = b.y;
			p[6] = b.z;
			p[7] = im.x;
			p[8] = im.y;
			p[9] = im.z;
			p[10] = im.w;
		}
		m += 1;
	}
	return m;
}

extern "C" F2D_API int32_t f2d_world_shape_capacity( int32_t worldId )
{
	HostWorld* W = world_from_id( worldId );
	return W ? W->shapeCount : 0;
}

extern "C" F2D_API int32_t f2d_world_get_shapes( int32_t worldId, float* floats, int32_t* ints, int32_t cap )
{
	HostWorld* W = world_from_id( worldId );
	if ( W == nullptr )
		return 0;
	cudaStreamSynchronize( W->stream );
	int n = std::min( W->shapeCount, cap );
	int up = std::min( n, W->shapeUploaded );
	std::vector<float4> aabb( W->aabb.begin(), W->aabb.begin() + n ), fat( W->fat.begin(), W->fat.begin() + n );
	std::vector<int> fl( W->sflags.begin(), W->sflags.begin() + n );
	if ( up > 0 )
	{
		cudaMemcpy( aabb.data(), W->d.aabb, sizeof( float4 ) * up, cudaMemcpyDeviceToHost );
		cudaMemcpy( fat.data(), W->d.fat, sizeof( float4 ) * up, cudaMemcpyDeviceToHost );
		cudaMemcpy( fl.data(), W->d.sflags, sizeof( int ) * up, cudaMemcpyDeviceToHost );
	}
	for ( int i = 0; i < n; ++i )
	{
		float* f = floats + 8 * i;
		f[0] = aabb[i].x;
		f[1] = aabb[i].y;
		f[2] = aabb[i].z;
		f[3] = aabb[i].w;
		f[4] = fat[i].x;
		f[5] = fat[i].y;
		f[6] = fat[i].z;
		f[7] = fat[i].w;
		int* k = ints + 4 * i;
		k[0] = W->proxyKey[i];
		k[1] = W->shapeBody[i];
		k[2] = shape_type( W->sflags[i] );
		k[3] = fl[i];
	}
	return n;
}

extern "C" F2D_API int32_t f2d_world_get_mass( int32_t worldId, float* out, int32_t cap )
{
	HostWorld* W = world_from_id( worldId );
	if ( W == nullptr )
		return 0;
	int n = std::min( W->bodyCount, cap );
	for ( int i = 0; i < n; ++i )
	{
		float* o = out + 8 * i;
		o[0] = W->bmass[i];
		o[1] = W->binertia[i];
		o[2] = W->massv[i].x;
		o[3] = W->massv[i].y;
		o[4] = W->localCenter[i].x;
		o[5] = W->localCenter[i].y;
		o[6] = W->massv[i].z;
		o[7] = W->massv[i].w;
	}
	return n;
}

// Contacts per graph colour as they stand now (the counts of the solver's
// stage set-up predate the islands that fell asleep at the end of the step).
__global__ void k_color_census( DWorld w, int* out12 )
{
	__shared__ int cnt[12];
	if ( threadIdx.x < 12 )
		cnt[threadIdx.x] = 0;
	__syncthreads();
	int n = w.sc->contactIdCount;
	for ( int c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x )
	{
		int col = w.ccolor[c];
		if ( col >= 0 && col < 12 && ( w.cflags[c] & CF_USED ) )
			atomicAdd( cnt + col, 1 );
	}
	__syncthreads();
	if ( threadIdx.x < 12 && cnt[threadIdx.x] > 0 )
		atomicAdd( out12 + threadIdx.x, cnt[threadIdx.x] );
}

extern "C" F2D_API void f2d_world_get_color_counts( int32_t worldId, int32_t* out12 )
{
	HostWorld* W = world_from_id( worldId );
	for ( int i = 0; i < 12; ++i )
		out12[i] = 0;
	if ( W == nullptr )
		return;
	flush_uploads( W );
	int* dOut = W->s.tmpA;
	cudaMemsetAsync( dOut, 0, sizeof( int ) * 12, W->stream );
	k_color_census<<<grid_for( W->d.contactCap ), 256, 0, W->stream>>>( W->d, dOut );
	cudaMemcpyAsync( out12, dOut, sizeof( int ) * 12, cudaMemcpyDeviceToHost, W->stream );
	cudaStreamSynchronize( W->stream );
	if ( W->jointCount > 0 )
	{
		std::vector<int> jc( W->jointCount );
		cudaMemcpy( jc.data(), W->d.jcolor, sizeof( int ) * W->jointCount, cudaMemcpyDeviceToHost );
		for ( int c : jc )
			if ( c >= 0 && c < 12 )
				out12[c] += 1;
	}
}

// ---------------------------------------------------------------------------
// events
// ---------------------------------------------------------------------------
extern "C" F2D_API void f2d_world_get_event_counts( int32_t worldId, int32_t* counts4 )
{
	HostWorld* W = world_from_id( worldId );
	for ( int i = 0; i < 4; ++i )
		counts4[i] = 0;
	if ( W == nullptr || !W->stepped )
		return;
	cudaStreamSynchronize( W->stream );
	DScalars sc;
	cudaMemcpy( &sc, W->d.sc, sizeof( sc ), cudaMemcpyDeviceToHost );
	int prefix = (int)W->endPrefix.size() / 4;
	if ( W->eventsCleared )
	{
		counts4[1] = prefix;
		return;
	}
	counts4[0] = sc.beginCount;
	counts4[1] = prefix + sc.endCount;
	counts4[2] = std::min( sc.hitCount, W->d.eventCap );
	int moved = 0;
	if ( W->islOn && W->islDev )
		cudaMemcpy( &moved, &W->islDev->moveCount, sizeof( int ), cudaMemcpyDeviceToHost );
	else
		moved = (int)W->awakeOrder.size();
	counts4[3] = moved;
}

static int read_pairs( HostWorld* W, const int* dptr, int count, int32_t* out4, int cap )
{
	int n = std::min( count, cap );
	std::vector<int> tmp( 2 * (size_t)n );
	if ( n > 0 )
		cudaMemcpy( tmp.data(), dptr, sizeof( int ) * 2 * n, cudaMemcpyDeviceToHost );
	for ( int i = 0; i < n; ++i )
	{
		int a = tmp[2 * i], b = tmp[2 * i + 1];
		out4[4 * i + 0] = a + 1;
		out4[4 * i + 1] = pack_wg( W, W->sgen[a] );
		out4[4 * i + 2] = b + 1;
		out4[4 * i + 3] = pack_wg( W, W->sgen[b] );
	}
	return n;
}

// b2World_GetSensorEvents (world.c:1505-1527; RawBox2D.worldGetSensorEvents, raw_box2d.dart:1295):
// this step's begin events (sensor shape, visitor shape) as id pairs, four
// ints per event; the end events likewise into end4, their count in
// *endCount. Returns the begin count.
extern "C" F2D_API int32_t f2d_world_get_sensor_events( int32_t worldId, int32_t* begin4, int32_t* end4, int32_t cap,
														 int32_t* endCount )
{
	if ( endCount )
		*endCount = 0;
	HostWorld* W = world_from_id( worldId );
	if ( W == nullptr || !W->stepped )
		return 0;
	// end events of sensors destroyed before the step come first
	int prefix = std::min( (int)W->sensorEndPrefix.size() / 4, (int)cap );
	std::copy( W->sensorEndPrefix.begin(), W->sensorEndPrefix.begin() + 4 * (size_t)prefix, end4 );
	if ( endCount )
		*endCount = prefix;
	if ( W->d.sensorCount == 0 || W->eventsCleared )
		return 0;
	cudaStreamSynchronize( W->stream );
	DScalars sc;
	cudaMemcpy( &sc, W->d.sc, sizeof( sc ), cudaMemcpyDeviceToHost );
	int nb = read_pairs( W, (const int*)W->d.sensorBeginEv, sc.sensorBegin, begin4, cap );
	int ne = read_pairs( W, (const int*)W->d.sensorEndEv, sc.sensorEnd, end4 + 4 * (size_t)prefix, cap - prefix );
	if ( endCount )
		*endCount = prefix + ne;
	return nb;
}

extern "C" F2D_API int32_t f2d_world_get_begin_events( int32_t worldId, int32_t* out4, int32_t cap )
{
	HostWorld* W = world_from_id( worldId );
	if ( W == nullptr || !W->stepped )
		return 0;
	int c[4];
	f2d_world_get_event_counts( worldId, c );
	return read_pairs( W, W->d.beginEv, c[0], out4, cap );
}

// The manifolds of the begin events (RawContactBeginEvent's normal and
// points, raw_box2d_ffi.dart:2205-2228, from b2ContactBeginTouchEvent.
// manifold): 9 floats per event in the order of f2d_world_get_begin_events.
extern "C" F2D_API int32_t f2d_world_get_begin_manifolds( int32_t worldId, float* out9, int32_t cap )
{
	HostWorld* W = world_from_id( worldId );
	if ( W == nullptr || !W->stepped )
		return 0;
	int c[4];
	f2d_world_get_event_counts( worldId, c );
	int n = std::min( c[0], cap );
	if ( n > 0 )
		cudaMemcpy( out9, W->d.beginEvF, sizeof( float ) * 9 * (size_t)n, cudaMemcpyDeviceToHost );
	return n;
}

extern "C" F2D_API int32_t f2d_world_get_end_events( int32_t worldId, int32_t* out4, int32_t cap )
{
	HostWorld* W = world_from_id( worldId );
	if ( W == nullptr || !W->stepped )
		return 0;
	int c[4];
	f2d_world_get_event_counts( worldId, c );
	int prefix = std::min( (int)W->endPrefix.size() / 4, (int)cap );
	std::copy( W->endPrefix.begin(), W->endPrefix.begin() + 4 * (size_t)prefix, out4 );
	return prefix + read_pairs( W, W->d.endEv, c[1] - (int)W->endPrefix.size() / 4, out4 + 4 * (size_t)prefix,
								cap - prefix );
}

extern "C" F2D_API int32_t f2d_world_get_hit_events( int32_t worldId, int32_t* ints4, float* floats5, int32_t cap )
{
	HostWorld* W = world_from_id( worldId );
	if ( W == nullptr || !W->stepped )
		return 0;
	int c[4];
	f2d_world_get_event_counts( worldId, c );
	int n = read_pairs( W, W->d.hitEvI, c[2], ints4, cap );
	if ( n > 0 )
		cudaMemcpy( floats5, W->d.hitEvF, sizeof( float ) * 5 * n, cudaMemcpyDeviceToHost );
	return n;
}

extern "C" F2D_API int32_t f2d_world_get_body_events( int32_t worldId, int32_t* ints3, float* floats4, int32_t cap )
{
	HostWorld* W = world_from_id( worldId );
	if ( W == nullptr || !W->stepped || W->eventsCleared )
		return 0;
	cudaStreamSynchronize( W->stream );
	int n = W->bodyCount;
	std::vector<float4> ev( n );
	if ( n > 0 )
		cudaMemcpy( ev.data(), W->d.moveEvXf, sizeof( float4 ) * n, cudaMemcpyDeviceToHost );
	if ( W->islOn && W->islDev )
	{
		// awake-set order with the fellAsleep flags (solver.c:603-611, solver_set.c:202-212)
		int count = 0;
		cudaMemcpy( &count, &W->islDev->moveCount, sizeof( int ), cudaMemcpyDeviceToHost );
		count = std::min( count, (int)cap );
		std::vector<int> mb( std::max( count, 1 ) ), ma( std::max( count, 1 ) );
		if ( count > 0 )
		{
			cudaMemcpy( mb.data(), W->islHost.moveBody, sizeof( int ) * count, cudaMemcpyDeviceToHost );
			cudaMemcpy( ma.data(), W->islHost.moveAsleep, sizeof( int ) * count, cudaMemcpyDeviceToHost );
		}
		for ( int i = 0; i < count; ++i )
		{
			int b = mb[i];
			ints3[3 * i + 0] = b + 1;
			ints3[3 * i + 1] = pack_wg( W, W->bgen[b] );
			ints3[3 * i + 2] = ma[i];
			floats4[4 * i + 0] = ev[b].x;
			floats4[4 * i + 1] = ev[b].y;
			floats4[4 * i + 2] = ev[b].z;
			floats4[4 * i + 3] = ev[b].w;
		}
		return count;
	}
	// the awake set's order (solver.c:603-611)
	int m = 0;
	for ( int b : W->awakeOrder )
	{
		if ( m >= cap )
			break;
		ints3[3 * m + 0] = b + 1;
		ints3[3 * m + 1] = pack_wg( W, W->bgen[b] );
		ints3[3 * m + 2] = 0;
		floats4[4 * m + 0] = ev[b].x;
		floats4[4 * m + 1] = ev[b].y;
		floats4[4 * m + 2] = ev[b].z;
		floats4[4 * m + 3] = ev[b].w;
		m += 1;
	}
	return m;
}

// ---------------------------------------------------------------------------
// profiling and counters
// ---------------------------------------------------------------------------
extern "C" F2D_API void f2d_world_set_profiling( int32_t worldId, int32_t enabled )
{
	HostWorld* W = world_from_id( worldId );
	if ( W == nullptr )
		return;
	W->profiling = enabled != 0;
}

extern "C" F2D_API void f2d_world_get_phase_ms( int32_t worldId, double* out6 )
{
	for ( int i = 0; i < 6; ++i )
		out6[i] = 0.0;
	HostWorld* W = world_from_id( worldId );
	if ( W == nullptr || W->ph[0] == nullptr )
		return;
	cudaStreamSynchronize( W->stream );
	// broadphase, narrowphase, colouring, solver set-up, solver kernel, finalize
	const int a[6] = { 0, 1, 2, 3, 4, 5 };
	const int b[6] = { 1, 2, 3, 4, 5, 6 };
	for ( int i = 0; i < 6; ++i )
	{
		float ms = 0.0f;
		if ( cudaEventElapsedTime( &ms, W->ph[a[i]], W->ph[b[i]] ) == cudaSuccess )
			out6[i] = ms;
	}
}

extern "C" F2D_API double f2d_world_get_rebuild_ms( int32_t worldId )
{
	HostWorld* W = world_from_id( worldId );
	if ( W == nullptr || W->ph[7] == nullptr )
		return 0.0;
	cudaStreamSynchronize( W->stream );
	float ms = 0.0f;
	if ( cudaEventElapsedTime( &ms, W->ph[7], W->ph[8] ) != cudaSuccess )
		return 0.0;
	return ms;
}

extern "C" F2D_API void f2d_world_get_counters( int32_t worldId, int32_t* out8 )
{
	for ( int i = 0; i < 8; ++i )
		out8[i] = 0;
	HostWorld* W = world_from_id( worldId );
	if ( W == nullptr )
		return;
	cudaStreamSynchronize( W->stream );
	DScalars sc;
	cudaMemcpy( &sc, W->d.sc, sizeof( sc ), cudaMemcpyDeviceToHost );
	int awake = 0;
	if ( W->islOn && W->islDev )
		cudaMemcpy( &awake, &W->islDev->awakeBodyCount, sizeof( int ), cudaMemcpyDeviceToHost );
	else
		awake = (int)W->awakeOrder.size();
	int active = 0;
	for ( int c = 0; c < 11; ++c )
		active += sc.colorCount[c] > 0 ? 1 : 0;
	out8[0] = awake;
	out8[1] = sc.contactIdCount - sc.contactFreeCount;
	out8[2] = sc.touchingCount;
	out8[3] = sc.overflowCount;
	out8[4] = active;
	out8[5] = sc.colorRounds;
	out8[6] = W->shapeCount - (int)W->shapeFree.size();
	out8[7] = W->jointCount - (int)W->jointFree.size();
}

// Latency side of the solver's roofline: the grid barriers the last
// grid-wide solver launch passed (0 after a cluster-solver step) and the
// measured cost of one barrier on its grid (n barriers timed by events).
extern "C" F2D_API void f2d_world_get_solver_latency( int32_t worldId, int32_t probeBarriers, double* out2 )
{
	out2[0] = out2[1] = 0.0;
	HostWorld* W = world_from_id( worldId );
	if ( W == nullptr )
		return;
	cudaStreamSynchronize( W->stream );
	int barriers = 0;
	cudaMemcpy( &barriers, &W->d.sc->solveBarriers, sizeof( int ), cudaMemcpyDeviceToHost );
	out2[0] = barriers;
	if ( probeBarriers > 0 && W->s.solverBlocks > 0 )
	{
		int* err = W->s.tmpB;
		cudaMemsetAsync( err, 0, sizeof( int ), W->stream );
		out2[1] = solver_barrier_probe( W->s, W->stream, (unsigned*)W->s.tmpA, err, probeBarriers );
	}
}

// ---------------------------------------------------------------------------
// accessors for queries.cu
// ---------------------------------------------------------------------------
DWorld* f2d_internal_world( int32_t worldId, cudaStream_t* st, int* gens, int genCap )
{
	(void)gens;
	(void)genCap;
	HostWorld* W = world_from_id( worldId );
	if ( W == nullptr )
		return nullptr;
	flush_uploads( W );
	cudaStreamSynchronize( W->stream );
	*st = W->stream;
	return &W->d;
}

// For the allocation-free queries: the world's device rows after pending
// uploads, or nullptr with *code set when serving them would need an
// allocation (capacities exceeded since the last step) or the world has more
// shapes than the caller's scratch holds. Uploads themselves only copy.
DWorld* f2d_internal_world_noalloc( int32_t worldId, cudaStream_t* st, int maxShapes, int* code )
{
	*code = 0;
	HostWorld* W = world_from_id( worldId );
	if ( W == nullptr )
		return nullptr;
	if ( W->shapeCount > maxShapes )
	{
		*code = F2D_NOALLOC_TOO_MANY_SHAPES;
		return nullptr;
	}
	const DWorld& d = W->d;
	// every path of flush_uploads that would allocate device memory: grown
	// body, shape or joint rows, a changed sensor list (its buffers are
	// reallocated), a broadphase tree whose node pool grew, rebuild scratch
	bool grows = W->bodyCount > d.bodyCap || W->shapeCount > d.shapeCap || W->jointCount > d.jointCap;
	grows = grows || W->sensorsDirty;
	for ( int t = 0; t < 3; ++t )
		grows = grows || ( W->treeDirty[t] && W->trees[t].cap > d.pt[t].cap );
	grows = grows || std::max( W->trees[1].cap, W->trees[2].cap ) > d.rb.cap;
	if ( grows )
	{
		*code = F2D_NOALLOC_NEEDS_GROWTH;
		return nullptr;
	}
	flush_uploads( W );
	cudaStreamSynchronize( W->stream );
	*st = W->stream;
	return &W->d;
}

uint16_t f2d_internal_shape_gen( int32_t worldId, int shape )
{
	HostWorld* W = world_from_id( worldId );
	if ( W == nullptr || shape < 0 || shape >= (int)W->sgen.size() )
		return 0;
	return W->sgen[shape];
}

int32_t f2d_internal_world0( int32_t worldId )
{
	HostWorld* W = world_from_id( worldId );
	return W ? W->index : 0;
}
