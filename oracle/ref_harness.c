// Flat C harness over the unmodified Box2D v3.1.1 sources vendored by forge2d
// (packages/forge2d/third_party/box2d). TEST INFRASTRUCTURE ONLY: this file is
// compiled together with the reference's own src/*.c into oracle/_ref/ by
// oracle/Makefile, and is loaded by tests/ and by bench.py's reference arm to
// pin the CPU restatement in oracle/port/ and to time the reference on the
// host cores. Nothing in the product links it.
//
// It exposes the same flat entry points as the restatement (prefix ref_ here,
// orc_ there) so a Python scene builder can drive both identically. Internal
// state (contacts, colours, manifolds) is read through the reference's private
// headers (world.h, contact.h, shape.h, body.h, constraint_graph.h).

#include "box2d/box2d.h"
#include "body.h"
#include "constraint_graph.h"
#include "contact.h"
#include "joint.h"
#include "shape.h"
#include "solver_set.h"
#include "world.h"

#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "port/f2d_defs.h"

// ---------------------------------------------------------------------------
// Persistent pthread pool behind b2EnqueueTaskCallback / b2FinishTaskCallback.
// forge2d itself never sets these (raw_box2d_ffi.dart:67-94 leaves workerCount
// at 1); the pool exists so the reference can be timed multithreaded.
// ---------------------------------------------------------------------------
#define POOL_MAX_THREADS 64
#define POOL_MAX_TASKS 256

typedef struct PoolTask
{
	b2TaskCallback* fcn;
	void* ctx;
	int itemCount;
	int minRange;
	int blockCount;
	int blockSize;
	volatile int nextBlock;
	volatile int doneBlocks;
	int used;
} PoolTask;

typedef struct Pool
{
	int threadCount; // including the caller
	pthread_t threads[POOL_MAX_THREADS];
	pthread_mutex_t mutex;
	pthread_cond_t cond;
	PoolTask tasks[POOL_MAX_TASKS];
	int taskHead;
	volatile int generation;
	volatile int quit;
} Pool;

static void pool_run_blocks( PoolTask* t, uint32_t workerIndex )
{
	while ( 1 )
	{
		int b = __atomic_fetch_add( &t->nextBlock, 1, __ATOMIC_ACQ_REL );
		if ( b >= t->blockCount )
			break;
		int start = b * t->blockSize;
		int end = start + t->blockSize;
		if ( end > t->itemCount )
			end = t->itemCount;
		t->fcn( start, end, workerIndex, t->ctx );
		__atomic_fetch_add( &t->doneBlocks, 1, __ATOMIC_ACQ_REL );
	}
}

typedef struct WorkerArg
{
	Pool* pool;
	int index;
} WorkerArg;

static WorkerArg s_workerArgs[POOL_MAX_THREADS];

static void* pool_worker( void* arg )
{
	WorkerArg* wa = arg;
	Pool* pool = wa->pool;
	int seenGen = 0;
	while ( 1 )
	{
		pthread_mutex_lock( &pool->mutex );
		while ( pool->generation == seenGen && pool->quit == 0 )
			pthread_cond_wait( &pool->cond, &pool->mutex );
		seenGen = pool->generation;
		int quit = pool->quit;
		pthread_mutex_unlock( &pool->mutex );
		if ( quit )
			break;
		// scan all tasks for blocks
		for ( int i = 0; i < POOL_MAX_TASKS; ++i )
		{
			PoolTask* t = pool->tasks + i;
			if ( __atomic_load_n( &t->used, __ATOMIC_ACQUIRE ) )
				pool_run_blocks( t, (uint32_t)wa->index );
		}
	}
	return NULL;
}

static void* pool_enqueue( b2TaskCallback* task, int itemCount, int minRange, void* taskContext, void* userContext )
{
	Pool* pool = userContext;
	if ( pool->threadCount <= 1 )
	{
		task( 0, itemCount, 0, taskContext );
		return NULL;
	}
	int slot = -1;
	pthread_mutex_lock( &pool->mutex );
	for ( int k = 0; k < POOL_MAX_TASKS; ++k )
	{
		int i = ( pool->taskHead + k ) % POOL_MAX_TASKS;
		if ( pool->tasks[i].used == 0 )
		{
			slot = i;
			pool->taskHead = ( i + 1 ) % POOL_MAX_TASKS;
			break;
		}
	}
	if ( slot < 0 )
	{
		pthread_mutex_unlock( &pool->mutex );
		task( 0, itemCount, (uint32_t)( pool->threadCount - 1 ), taskContext );
		return NULL;
	}
	PoolTask* t = pool->tasks + slot;
	int blocks = pool->threadCount * 4;
	int blockSize = ( itemCount + blocks - 1 ) / blocks;
	if ( blockSize < minRange )
		blockSize = minRange;
	if ( blockSize < 1 )
		blockSize = 1;
	t->fcn = task;
	t->ctx = taskContext;
	t->itemCount = itemCount;
	t->minRange = minRange;
	t->blockSize = blockSize;
	t->blockCount = ( itemCount + blockSize - 1 ) / blockSize;
	t->nextBlock = 0;
	t->doneBlocks = 0;
	__atomic_store_n( &t->used, 1, __ATOMIC_RELEASE );
	pool->generation += 1;
	pthread_cond_broadcast( &pool->cond );
	pthread_mutex_unlock( &pool->mutex );
	return t;
}

static void pool_finish( void* userTask, void* userContext )
{
	PoolTask* t = userTask;
	if ( t == NULL )
		return;
	Pool* pool = userContext;
	// The calling thread helps with any pending block (its own task first)
	// until this task is complete; the solver's worker-0 task waits on the
	// other workers, so an unclaimed worker task must never be left idle.
	uint32_t me = (uint32_t)( pool->threadCount - 1 );
	pool_run_blocks( t, me );
	while ( __atomic_load_n( &t->doneBlocks, __ATOMIC_ACQUIRE ) < t->blockCount )
	{
		for ( int i = 0; i < POOL_MAX_TASKS; ++i )
		{
			PoolTask* o = pool->tasks + i;
			if ( o != t && __atomic_load_n( &o->used, __ATOMIC_ACQUIRE ) &&
				 __atomic_load_n( &o->nextBlock, __ATOMIC_ACQUIRE ) < o->blockCount )
				pool_run_blocks( o, me );
		}
	}
	__atomic_store_n( &t->used, 0, __ATOMIC_RELEASE );
}

static Pool* pool_create( int threadCount )
{
	Pool* pool = calloc( 1, sizeof( Pool ) );
	pool->threadCount = threadCount;
	pthread_mutex_init( &pool->mutex, NULL );
	pthread_cond_init( &pool->cond, NULL );
	// worker indices 0..threadCount-2 for pool threads; the calling thread
	// uses threadCount-1 when it helps in pool_finish
	for ( int i = 0; i < threadCount - 1; ++i )
	{
		s_workerArgs[i].pool = pool;
		s_workerArgs[i].index = i;
		pthread_create( pool->threads + i, NULL, pool_worker, s_workerArgs + i );
	}
	return pool;
}

static void pool_destroy( Pool* pool )
{
	if ( pool == NULL )
		return;
	pthread_mutex_lock( &pool->mutex );
	pool->quit = 1;
	pool->generation += 1;
	pthread_cond_broadcast( &pool->cond );
	pthread_mutex_unlock( &pool->mutex );
	for ( int i = 0; i < pool->threadCount - 1; ++i )
		pthread_join( pool->threads[i], NULL );
	free( pool );
}

// ---------------------------------------------------------------------------
// World table
// ---------------------------------------------------------------------------
#define REF_MAX_WORLDS 64
static b2WorldId s_worlds[REF_MAX_WORLDS];
static Pool* s_pools[REF_MAX_WORLDS];
static int s_used[REF_MAX_WORLDS];

static b2World* ref_world( int w )
{
	return b2GetWorldFromId( s_worlds[w] );
}

int ref_create_world( const f2d_world_def* d, int workerCount )
{
	int slot = -1;
	for ( int i = 0; i < REF_MAX_WORLDS; ++i )
	{
		if ( s_used[i] == 0 )
		{
			slot = i;
			break;
		}
	}
	if ( slot < 0 )
		return -1;
	b2WorldDef def = b2DefaultWorldDef();
	def.gravity = ( b2Vec2 ){ (float)d->gravityX, (float)d->gravityY };
	def.restitutionThreshold = (float)d->restitutionThreshold;
	def.hitEventThreshold = (float)d->hitEventThreshold;
	def.contactHertz = (float)d->contactHertz;
	def.contactDampingRatio = (float)d->contactDampingRatio;
	def.maxContactPushSpeed = (float)d->maxContactPushSpeed;
	def.maximumLinearSpeed = (float)d->maximumLinearSpeed;
	def.enableSleep = d->enableSleep != 0;
	def.enableContinuous = d->enableContinuous != 0;
	s_pools[slot] = NULL;
	if ( workerCount > 1 )
	{
		if ( workerCount > POOL_MAX_THREADS )
			workerCount = POOL_MAX_THREADS;
		s_pools[slot] = pool_create( workerCount );
		def.workerCount = workerCount;
		def.enqueueTask = pool_enqueue;
		def.finishTask = pool_finish;
		def.userTaskContext = s_pools[slot];
	}
	s_worlds[slot] = b2CreateWorld( &def );
	s_used[slot] = 1;
	return slot;
}

void ref_destroy_world( int w )
{
	if ( w < 0 || w >= REF_MAX_WORLDS || s_used[w] == 0 )
		return;
	b2DestroyWorld( s_worlds[w] );
	pool_destroy( s_pools[w] );
	s_pools[w] = NULL;
	s_used[w] = 0;
}

void ref_world_step( int w, double dt, int subSteps )
{
	b2World_Step( s_worlds[w], (float)dt, subSteps );
}

double ref_world_step_timed( int w, double dt, int subSteps, int steps )
{
	struct timespec t0, t1;
	clock_gettime( CLOCK_MONOTONIC, &t0 );
	for ( int i = 0; i < steps; ++i )
		b2World_Step( s_worlds[w], (float)dt, subSteps );
	clock_gettime( CLOCK_MONOTONIC, &t1 );
	return ( t1.tv_sec - t0.tv_sec ) + 1e-9 * ( t1.tv_nsec - t0.tv_nsec );
}

int ref_create_body( int w, const f2d_body_def* d )
{
	b2BodyDef def = b2DefaultBodyDef();
	def.type = (b2BodyType)d->type;
	def.position = ( b2Vec2 ){ (float)d->positionX, (float)d->positionY };
	def.rotation = ( b2Rot ){ (float)d->rotationCos, (float)d->rotationSin };
	def.linearVelocity = ( b2Vec2 ){ (float)d->linearVelocityX, (float)d->linearVelocityY };
	def.angularVelocity = (float)d->angularVelocity;
	def.linearDamping = (float)d->linearDamping;
	def.angularDamping = (float)d->angularDamping;
	def.gravityScale = (float)d->gravityScale;
	def.sleepThreshold = (float)d->sleepThreshold;
	def.enableSleep = d->enableSleep != 0;
	def.isAwake = d->isAwake != 0;
	def.fixedRotation = d->fixedRotation != 0;
	def.isBullet = d->isBullet != 0;
	def.isEnabled = d->isEnabled != 0;
	def.allowFastRotation = d->allowFastRotation != 0;
	b2BodyId id = b2CreateBody( s_worlds[w], &def );
	return id.index1 - 1;
}

static b2BodyId ref_body_id( int w, int body )
{
	b2World* world = ref_world( w );
	b2Body* b = b2BodyArray_Get( &world->bodies, body );
	b2BodyId id = { body + 1, world->worldId, b->generation };
	return id;
}

static b2ShapeDef ref_shape_def( const f2d_shape_def* d )
{
	b2ShapeDef def = b2DefaultShapeDef();
	def.material.friction = (float)d->friction;
	def.material.restitution = (float)d->restitution;
	def.material.rollingResistance = (float)d->rollingResistance;
	def.material.tangentSpeed = (float)d->tangentSpeed;
	def.material.userMaterialId = d->userMaterialId;
	def.density = (float)d->density;
	def.filter.categoryBits = (uint64_t)d->categoryBits;
	def.filter.maskBits = (uint64_t)d->maskBits;
	def.filter.groupIndex = d->groupIndex;
	def.isSensor = d->isSensor != 0;
	def.enableSensorEvents = d->enableSensorEvents != 0;
	def.enableContactEvents = d->enableContactEvents != 0;
	def.enableHitEvents = d->enableHitEvents != 0;
	def.enablePreSolveEvents = d->enablePreSolveEvents != 0;
	def.invokeContactCreation = d->invokeContactCreation != 0;
	def.updateBodyMass = d->updateBodyMass != 0;
	return def;
}

int ref_create_circle_shape( int w, int body, const f2d_shape_def* d, double cx, double cy, double radius )
{
	b2ShapeDef def = ref_shape_def( d );
	b2Circle c = { { (float)cx, (float)cy }, (float)radius };
	b2ShapeId id = b2CreateCircleShape( ref_body_id( w, body ), &def, &c );
	return id.index1 - 1;
}

int ref_create_capsule_shape( int w, int body, const f2d_shape_def* d, double x1, double y1, double x2, double y2,
							  double radius )
{
	b2ShapeDef def = ref_shape_def( d );
	b2Capsule c = { { (float)x1, (float)y1 }, { (float)x2, (float)y2 }, (float)radius };
	b2ShapeId id = b2CreateCapsuleShape( ref_body_id( w, body ), &def, &c );
	return id.index1 - 1;
}

int ref_create_segment_shape( int w, int body, const f2d_shape_def* d, double x1, double y1, double x2, double y2 )
{
	b2ShapeDef def = ref_shape_def( d );
	b2Segment s = { { (float)x1, (float)y1 }, { (float)x2, (float)y2 } };
	b2ShapeId id = b2CreateSegmentShape( ref_body_id( w, body ), &def, &s );
	return id.index1 - 1;
}

int ref_create_chain( int w, int body, const double* points, int count, const double* materials, int materialCount,
					  long long categoryBits, long long maskBits, int groupIndex, int isLoop, int enableSensorEvents )
{
	b2Vec2* pts = (b2Vec2*)malloc( sizeof( b2Vec2 ) * (size_t)count );
	b2SurfaceMaterial* mats = (b2SurfaceMaterial*)malloc( sizeof( b2SurfaceMaterial ) * (size_t)materialCount );
	for ( int i = 0; i < count; ++i )
		pts[i] = ( b2Vec2 ){ (float)points[2 * i], (float)points[2 * i + 1] };
	for ( int i = 0; i < materialCount; ++i )
	{
		const double* m = materials + 6 * i;
		mats[i] = ( b2SurfaceMaterial ){ 0 };
		mats[i].friction = (float)m[0];
		mats[i].restitution = (float)m[1];
		mats[i].rollingResistance = (float)m[2];
		mats[i].tangentSpeed = (float)m[3];
		mats[i].userMaterialId = (int)m[4];
		mats[i].customColor = (uint32_t)m[5];
	}
	b2ChainDef def = b2DefaultChainDef();
	def.points = pts;
	def.count = count;
	def.materials = mats;
	def.materialCount = materialCount;
	def.filter.categoryBits = (uint64_t)categoryBits;
	def.filter.maskBits = (uint64_t)maskBits;
	def.filter.groupIndex = groupIndex;
	def.isLoop = isLoop != 0;
	def.enableSensorEvents = enableSensorEvents != 0;
	b2ChainId id = b2CreateChain( ref_body_id( w, body ), &def );
	free( pts );
	free( mats );
	return id.index1 - 1;
}

int ref_chain_get_segments( int w, int chain, int* out, int capacity )
{
	b2World* world = ref_world( w );
	b2ChainShape* ch = world->chainShapes.data + chain;
	int n = ch->count < capacity ? ch->count : capacity;
	for ( int i = 0; i < n; ++i )
		out[i] = ch->shapeIndices[i];
	return ch->count;
}

int ref_create_box_shape( int w, int body, const f2d_shape_def* d, double hx, double hy, double cx, double cy,
						  double c, double s, double radius )
{
	b2ShapeDef def = ref_shape_def( d );
	b2Polygon p = b2MakeOffsetRoundedBox( (float)hx, (float)hy, ( b2Vec2 ){ (float)cx, (float)cy },
										  ( b2Rot ){ (float)c, (float)s }, (float)radius );
	b2ShapeId id = b2CreatePolygonShape( ref_body_id( w, body ), &def, &p );
	return id.index1 - 1;
}

// points packed x0,y0,x1,y1,... Returns -1 for a degenerate hull (forge2d
// throws ArgumentError there, raw_box2d_ffi.dart:717-721).
int ref_create_polygon_shape( int w, int body, const f2d_shape_def* d, const double* points, int count, double radius )
{
	b2Vec2 v[B2_MAX_POLYGON_VERTICES];
	if ( count > B2_MAX_POLYGON_VERTICES )
		return -1;
	for ( int i = 0; i < count; ++i )
		v[i] = ( b2Vec2 ){ (float)points[2 * i], (float)points[2 * i + 1] };
	b2Hull hull = b2ComputeHull( v, count );
	if ( hull.count == 0 )
		return -1;
	b2Polygon p = b2MakePolygon( &hull, (float)radius );
	b2ShapeDef def = ref_shape_def( d );
	b2ShapeId id = b2CreatePolygonShape( ref_body_id( w, body ), &def, &p );
	return id.index1 - 1;
}

int ref_create_revolute_joint( int w, const f2d_revolute_def* d )
{
	b2RevoluteJointDef def = b2DefaultRevoluteJointDef();
	def.bodyIdA = ref_body_id( w, d->bodyA );
	def.bodyIdB = ref_body_id( w, d->bodyB );
	def.localAnchorA = ( b2Vec2 ){ (float)d->localAnchorAX, (float)d->localAnchorAY };
	def.localAnchorB = ( b2Vec2 ){ (float)d->localAnchorBX, (float)d->localAnchorBY };
	def.referenceAngle = (float)d->referenceAngle;
	def.targetAngle = (float)d->targetAngle;
	def.enableSpring = d->enableSpring != 0;
	def.hertz = (float)d->hertz;
	def.dampingRatio = (float)d->dampingRatio;
	def.enableLimit = d->enableLimit != 0;
	def.lowerAngle = (float)d->lowerAngle;
	def.upperAngle = (float)d->upperAngle;
	def.enableMotor = d->enableMotor != 0;
	def.maxMotorTorque = (float)d->maxMotorTorque;
	def.motorSpeed = (float)d->motorSpeed;
	def.drawSize = (float)d->drawSize;
	def.collideConnected = d->collideConnected != 0;
	b2JointId id = b2CreateRevoluteJoint( s_worlds[w], &def );
	return id.index1 - 1;
}

// Weld and distance joints (b2CreateWeldJoint, b2CreateDistanceJoint)
int ref_create_joint( int w, const f2d_joint_def* d )
{
	b2JointId id = { 0 };
	b2Vec2 la = { (float)d->localAnchorAX, (float)d->localAnchorAY };
	b2Vec2 lb = { (float)d->localAnchorBX, (float)d->localAnchorBY };
	if ( d->type == F2D_JOINT_WELD )
	{
		b2WeldJointDef def = b2DefaultWeldJointDef();
		def.bodyIdA = ref_body_id( w, d->bodyA );
		def.bodyIdB = ref_body_id( w, d->bodyB );
		def.localAnchorA = la;
		def.localAnchorB = lb;
		def.referenceAngle = (float)d->referenceAngle;
		def.linearHertz = (float)d->linearHertz;
		def.linearDampingRatio = (float)d->linearDampingRatio;
		def.angularHertz = (float)d->angularHertz;
		def.angularDampingRatio = (float)d->angularDampingRatio;
		def.collideConnected = d->collideConnected != 0;
		id = b2CreateWeldJoint( s_worlds[w], &def );
	}
	else if ( d->type == F2D_JOINT_DISTANCE )
	{
		b2DistanceJointDef def = b2DefaultDistanceJointDef();
		def.bodyIdA = ref_body_id( w, d->bodyA );
		def.bodyIdB = ref_body_id( w, d->bodyB );
		def.localAnchorA = la;
		def.localAnchorB = lb;
		def.length = (float)d->length;
		def.minLength = (float)d->minLength;
		def.maxLength = (float)d->maxLength;
		def.hertz = (float)d->hertz;
		def.dampingRatio = (float)d->dampingRatio;
		def.maxMotorForce = (float)d->maxMotorForce;
		def.motorSpeed = (float)d->motorSpeed;
		def.enableSpring = d->enableSpring != 0;
		def.enableLimit = d->enableLimit != 0;
		def.enableMotor = d->enableMotor != 0;
		def.collideConnected = d->collideConnected != 0;
		id = b2CreateDistanceJoint( s_worlds[w], &def );
	}
	else if ( d->type == F2D_JOINT_PRISMATIC )
	{
		b2PrismaticJointDef def = b2DefaultPrismaticJointDef();
		def.bodyIdA = ref_body_id( w, d->bodyA );
		def.bodyIdB = ref_body_id( w, d->bodyB );
		def.localAnchorA = la;
		def.localAnchorB = lb;
		def.localAxisA = ( b2Vec2 ){ (float)d->localAxisAX, (float)d->localAxisAY };
		def.referenceAngle = (float)d->referenceAngle;
		def.targetTranslation = (float)d->targetTranslation;
		def.enableSpring = d->enableSpring != 0;
		def.hertz = (float)d->hertz;
		def.dampingRatio = (float)d->dampingRatio;
		def.enableLimit = d->enableLimit != 0;
		def.lowerTranslation = (float)d->lowerTranslation;
		def.upperTranslation = (float)d->upperTranslation;
		def.enableMotor = d->enableMotor != 0;
		def.maxMotorForce = (float)d->maxMotorForce;
		def.motorSpeed = (float)d->motorSpeed;
		def.collideConnected = d->collideConnected != 0;
		id = b2CreatePrismaticJoint( s_worlds[w], &def );
	}
	else if ( d->type == F2D_JOINT_WHEEL )
	{
		b2WheelJointDef def = b2DefaultWheelJointDef();
		def.bodyIdA = ref_body_id( w, d->bodyA );
		def.bodyIdB = ref_body_id( w, d->bodyB );
		def.localAnchorA = la;
		def.localAnchorB = lb;
		def.localAxisA = ( b2Vec2 ){ (float)d->localAxisAX, (float)d->localAxisAY };
		def.enableSpring = d->enableSpring != 0;
		def.hertz = (float)d->hertz;
		def.dampingRatio = (float)d->dampingRatio;
		def.enableLimit = d->enableLimit != 0;
		def.lowerTranslation = (float)d->lowerTranslation;
		def.upperTranslation = (float)d->upperTranslation;
		def.enableMotor = d->enableMotor != 0;
		def.maxMotorTorque = (float)d->maxMotorTorque;
		def.motorSpeed = (float)d->motorSpeed;
		def.collideConnected = d->collideConnected != 0;
		id = b2CreateWheelJoint( s_worlds[w], &def );
	}
	else if ( d->type == F2D_JOINT_MOTOR )
	{
		b2MotorJointDef def = b2DefaultMotorJointDef();
		def.bodyIdA = ref_body_id( w, d->bodyA );
		def.bodyIdB = ref_body_id( w, d->bodyB );
		def.linearOffset = ( b2Vec2 ){ (float)d->linearOffsetX, (float)d->linearOffsetY };
		def.angularOffset = (float)d->angularOffset;
		def.maxForce = (float)d->maxForce;
		def.maxTorque = (float)d->maxTorque;
		def.correctionFactor = (float)d->correctionFactor;
		def.collideConnected = d->collideConnected != 0;
		id = b2CreateMotorJoint( s_worlds[w], &def );
	}
	else if ( d->type == F2D_JOINT_MOUSE )
	{
		b2MouseJointDef def = b2DefaultMouseJointDef();
		def.bodyIdA = ref_body_id( w, d->bodyA );
		def.bodyIdB = ref_body_id( w, d->bodyB );
		def.target = ( b2Vec2 ){ (float)d->targetX, (float)d->targetY };
		def.hertz = (float)d->hertz;
		def.dampingRatio = (float)d->dampingRatio;
		def.maxForce = (float)d->maxForce;
		def.collideConnected = d->collideConnected != 0;
		id = b2CreateMouseJoint( s_worlds[w], &def );
	}
	else if ( d->type == F2D_JOINT_FILTER )
	{
		b2FilterJointDef def = b2DefaultFilterJointDef();
		def.bodyIdA = ref_body_id( w, d->bodyA );
		def.bodyIdB = ref_body_id( w, d->bodyB );
		id = b2CreateFilterJoint( s_worlds[w], &def );
	}
	else
		return -1;
	return id.index1 - 1;
}

void ref_mouse_joint_set_target( int w, int j, double x, double y )
{
	b2World* world = ref_world( w );
	b2Joint* joint = b2JointArray_Get( &world->joints, j );
	b2JointId id = { j + 1, world->worldId, joint->generation };
	b2MouseJoint_SetTarget( id, ( b2Vec2 ){ (float)x, (float)y } );
}

int ref_get_sensor_events( int w, int* begin, int* end, int cap, int* endCount )
{
	b2SensorEvents ev = b2World_GetSensorEvents( s_worlds[w] );
	for ( int i = 0; i < ev.beginCount && i < cap; ++i )
	{
		begin[2 * i] = ev.beginEvents[i].sensorShapeId.index1 - 1;
		begin[2 * i + 1] = ev.beginEvents[i].visitorShapeId.index1 - 1;
	}
	for ( int i = 0; i < ev.endCount && i < cap; ++i )
	{
		end[2 * i] = ev.endEvents[i].sensorShapeId.index1 - 1;
		end[2 * i + 1] = ev.endEvents[i].visitorShapeId.index1 - 1;
	}
	*endCount = ev.endCount;
	return ev.beginCount;
}

void ref_joint_set_motor( int w, int j, int enable, double speed, double maxMotor )
{
	b2World* world = ref_world( w );
	b2Joint* joint = b2JointArray_Get( &world->joints, j );
	b2JointId id = { j + 1, world->worldId, joint->generation };
	switch ( b2Joint_GetType( id ) )
	{
		case b2_revoluteJoint:
			b2RevoluteJoint_EnableMotor( id, enable != 0 );
			b2RevoluteJoint_SetMotorSpeed( id, (float)speed );
			b2RevoluteJoint_SetMaxMotorTorque( id, (float)maxMotor );
			break;
		case b2_prismaticJoint:
			b2PrismaticJoint_EnableMotor( id, enable != 0 );
			b2PrismaticJoint_SetMotorSpeed( id, (float)speed );
			b2PrismaticJoint_SetMaxMotorForce( id, (float)maxMotor );
			break;
		case b2_wheelJoint:
			b2WheelJoint_EnableMotor( id, enable != 0 );
			b2WheelJoint_SetMotorSpeed( id, (float)speed );
			b2WheelJoint_SetMaxMotorTorque( id, (float)maxMotor );
			break;
		case b2_distanceJoint:
			b2DistanceJoint_EnableMotor( id, enable != 0 );
			b2DistanceJoint_SetMotorSpeed( id, (float)speed );
			b2DistanceJoint_SetMaxMotorForce( id, (float)maxMotor );
			break;
		default:
			break;
	}
}

void ref_joint_set_limits( int w, int j, int enable, double lower, double upper )
{
	b2World* world = ref_world( w );
	b2Joint* joint = b2JointArray_Get( &world->joints, j );
	b2JointId id = { j + 1, world->worldId, joint->generation };
	switch ( b2Joint_GetType( id ) )
	{
		case b2_revoluteJoint:
			b2RevoluteJoint_EnableLimit( id, enable != 0 );
			b2RevoluteJoint_SetLimits( id, (float)lower, (float)upper );
			break;
		case b2_prismaticJoint:
			b2PrismaticJoint_EnableLimit( id, enable != 0 );
			b2PrismaticJoint_SetLimits( id, (float)lower, (float)upper );
			break;
		case b2_wheelJoint:
			b2WheelJoint_EnableLimit( id, enable != 0 );
			b2WheelJoint_SetLimits( id, (float)lower, (float)upper );
			break;
		default:
			break;
	}
}

void ref_joint_get_constraint( int w, int j, float* out3 )
{
	b2World* world = ref_world( w );
	out3[0] = out3[1] = out3[2] = 0.0f;
	if ( j < 0 || j >= world->joints.count || world->joints.data[j].jointId != j )
		return;
	b2Joint* joint = b2JointArray_Get( &world->joints, j );
	b2JointId id = { j + 1, world->worldId, joint->generation };
	b2Vec2 f = b2Joint_GetConstraintForce( id );
	out3[0] = f.x;
	out3[1] = f.y;
	out3[2] = b2Joint_GetConstraintTorque( id );
}

typedef struct RefCast
{
	orc_cast_fn fn;
	void* context;
} RefCast;

static float ref_cast_trampoline( b2ShapeId id, b2Vec2 point, b2Vec2 normal, float fraction, void* context )
{
	RefCast* c = (RefCast*)context;
	return c->fn( id.index1 - 1, point.x, point.y, normal.x, normal.y, fraction, c->context );
}

// b2World_CastRay with the callback form (the reference's tree order)
int ref_world_cast_ray( int w, double ox, double oy, double tx, double ty, long long cat, long long mask, orc_cast_fn fn,
						void* context )
{
	RefCast c = { fn, context };
	b2QueryFilter f = { (uint64_t)cat, (uint64_t)mask };
	b2World_CastRay( s_worlds[w], ( b2Vec2 ){ (float)ox, (float)oy }, ( b2Vec2 ){ (float)tx, (float)ty }, f,
					 ref_cast_trampoline, &c );
	return 0;
}

void ref_world_explode( int w, long long maskBits, double px, double py, double radius, double falloff,
						double impulsePerLength )
{
	b2ExplosionDef def = b2DefaultExplosionDef();
	def.maskBits = (uint64_t)maskBits;
	def.position = ( b2Vec2 ){ (float)px, (float)py };
	def.radius = (float)radius;
	def.falloff = (float)falloff;
	def.impulsePerLength = (float)impulsePerLength;
	b2World_Explode( s_worlds[w], &def );
}

// user callbacks: b2World_SetCustomFilterCallback / SetPreSolveCallback
// with the 0-based shape ids and the manifold view of f2d_defs.h
typedef struct RefCallbacks
{
	orc_custom_filter_fn filter;
	void* filterContext;
	orc_pre_solve_fn preSolve;
	void* preSolveContext;
} RefCallbacks;
static RefCallbacks s_callbacks[REF_MAX_WORLDS];

static bool ref_filter_trampoline( b2ShapeId a, b2ShapeId b, void* context )
{
	RefCallbacks* cb = (RefCallbacks*)context;
	return cb->filter( a.index1 - 1, b.index1 - 1, cb->filterContext ) != 0;
}

static bool ref_pre_solve_trampoline( b2ShapeId a, b2ShapeId b, b2Manifold* m, void* context )
{
	RefCallbacks* cb = (RefCallbacks*)context;
	f2d_manifold_view mv;
	memset( &mv, 0, sizeof( mv ) );
	mv.normalX = m->normal.x;
	mv.normalY = m->normal.y;
	mv.pointCount = m->pointCount;
	for ( int i = 0; i < m->pointCount && i < 2; ++i )
	{
		const b2ManifoldPoint* mp = m->points + i;
		f2d_manifold_point_view* q = mv.points + i;
		q->pointX = mp->point.x;
		q->pointY = mp->point.y;
		q->anchorAX = mp->anchorA.x;
		q->anchorAY = mp->anchorA.y;
		q->anchorBX = mp->anchorB.x;
		q->anchorBY = mp->anchorB.y;
		q->separation = mp->separation;
		q->id = mp->id;
	}
	return cb->preSolve( a.index1 - 1, b.index1 - 1, &mv, cb->preSolveContext ) != 0;
}

void ref_set_custom_filter( int w, orc_custom_filter_fn fn, void* context )
{
	s_callbacks[w].filter = fn;
	s_callbacks[w].filterContext = context;
	b2World_SetCustomFilterCallback( s_worlds[w], fn ? ref_filter_trampoline : NULL, s_callbacks + w );
}

void ref_set_pre_solve( int w, orc_pre_solve_fn fn, void* context )
{
	s_callbacks[w].preSolve = fn;
	s_callbacks[w].preSolveContext = context;
	b2World_SetPreSolveCallback( s_worlds[w], fn ? ref_pre_solve_trampoline : NULL, s_callbacks + w );
}

// ---------------------------------------------------------------------------
// State dumps
// ---------------------------------------------------------------------------
int ref_body_capacity( int w )
{
	return ref_world( w )->bodies.count;
}

// Per body id: px py c s vx vy w cx cy (center of mass) | valid flag in out[9]
// Layout F2D_BODY_DUMP_STRIDE floats per body.
int ref_get_bodies( int w, float* out, int cap )
{
	b2World* world = ref_world( w );
	int n = world->bodies.count < cap ? world->bodies.count : cap;
	for ( int i = 0; i < n; ++i )
	{
		float* o = out + F2D_BODY_DUMP_STRIDE * i;
		memset( o, 0, sizeof( float ) * F2D_BODY_DUMP_STRIDE );
		b2Body* body = world->bodies.data + i;
		if ( body->id == B2_NULL_INDEX )
			continue;
		b2BodySim* sim = b2GetBodySim( world, body );
		b2BodyState* st = b2GetBodyState( world, body );
		o[0] = sim->transform.p.x;
		o[1] = sim->transform.p.y;
		o[2] = sim->transform.q.c;
		o[3] = sim->transform.q.s;
		if ( st )
		{
			o[4] = st->linearVelocity.x;
			o[5] = st->linearVelocity.y;
			o[6] = st->angularVelocity;
		}
		o[7] = sim->center.x;
		o[8] = sim->center.y;
		o[9] = 1.0f;
		o[10] = (float)body->setIndex;
		o[11] = body->sleepTime;
	}
	return n;
}

int ref_contact_capacity( int w )
{
	return ref_world( w )->contacts.count;
}

// Per live contact: ints [id, shapeA, shapeB, color, pointCount, flags, simFlags, id0, id1]
// floats [F2D_CONTACT_DUMP_FLOATS]: normal(2) rolling(1) then per point:
// anchorA(2) anchorB(2) point(2) separation normalImpulse tangentImpulse totalNormalImpulse normalVelocity
int ref_get_contacts( int w, int* ints, float* floats, int cap )
{
	b2World* world = ref_world( w );
	int n = 0;
	for ( int i = 0; i < world->contacts.count && n < cap; ++i )
	{
		b2Contact* c = world->contacts.data + i;
		if ( c->contactId == B2_NULL_INDEX )
			continue;
		b2ContactSim* sim = b2GetContactSim( world, c );
		int* oi = ints + F2D_CONTACT_DUMP_INTS * n;
		float* of = floats + F2D_CONTACT_DUMP_FLOATS * n;
		oi[0] = c->contactId;
		oi[1] = c->shapeIdA;
		oi[2] = c->shapeIdB;
		oi[3] = c->colorIndex;
		oi[4] = sim->manifold.pointCount;
		oi[5] = (int)c->flags;
		oi[6] = (int)sim->simFlags;
		oi[7] = sim->manifold.points[0].id;
		oi[8] = sim->manifold.points[1].id;
		of[0] = sim->manifold.normal.x;
		of[1] = sim->manifold.normal.y;
		of[2] = sim->manifold.rollingImpulse;
		for ( int k = 0; k < 2; ++k )
		{
			b2ManifoldPoint* mp = sim->manifold.points + k;
			float* p = of + 3 + 11 * k;
			p[0] = mp->anchorA.x;
			p[1] = mp->anchorA.y;
			p[2] = mp->anchorB.x;
			p[3] = mp->anchorB.y;
			p[4] = mp->point.x;
			p[5] = mp->point.y;
			p[6] = mp->separation;
			p[7] = mp->normalImpulse;
			p[8] = mp->tangentImpulse;
			p[9] = mp->totalNormalImpulse;
			p[10] = mp->normalVelocity;
		}
		n += 1;
	}
	return n;
}

int ref_shape_capacity( int w )
{
	return ref_world( w )->shapes.count;
}

// Per shape id: aabb(4) fatAABB(4) | ints: proxyKey, bodyId, type, enlarged
int ref_get_shapes( int w, float* floats, int* ints, int cap )
{
	b2World* world = ref_world( w );
	int n = world->shapes.count < cap ? world->shapes.count : cap;
	for ( int i = 0; i < n; ++i )
	{
		b2Shape* s = world->shapes.data + i;
		float* f = floats + 8 * i;
		int* k = ints + 4 * i;
		f[0] = s->aabb.lowerBound.x;
		f[1] = s->aabb.lowerBound.y;
		f[2] = s->aabb.upperBound.x;
		f[3] = s->aabb.upperBound.y;
		f[4] = s->fatAABB.lowerBound.x;
		f[5] = s->fatAABB.lowerBound.y;
		f[6] = s->fatAABB.upperBound.x;
		f[7] = s->fatAABB.upperBound.y;
		k[0] = s->proxyKey;
		k[1] = s->bodyId;
		k[2] = (int)s->type;
		k[3] = s->enlargedAABB ? 1 : 0;
	}
	return n;
}

// Body mass data per body id: mass, inertia, invMass, invInertia, localCenter(2), minExtent, maxExtent
int ref_get_mass( int w, float* out, int cap )
{
	b2World* world = ref_world( w );
	int n = world->bodies.count < cap ? world->bodies.count : cap;
	for ( int i = 0; i < n; ++i )
	{
		float* o = out + 8 * i;
		memset( o, 0, 8 * sizeof( float ) );
		b2Body* body = world->bodies.data + i;
		if ( body->id == B2_NULL_INDEX )
			continue;
		b2BodySim* sim = b2GetBodySim( world, body );
		o[0] = body->mass;
		o[1] = body->inertia;
		o[2] = sim->invMass;
		o[3] = sim->invInertia;
		o[4] = sim->localCenter.x;
		o[5] = sim->localCenter.y;
		o[6] = sim->minExtent;
		o[7] = sim->maxExtent;
	}
	return n;
}

// Polygon geometry as stored for a shape: count, radius, centroid(2), verts(16), normals(16)
int ref_get_polygon( int w, int shape, float* out )
{
	b2World* world = ref_world( w );
	b2Shape* s = world->shapes.data + shape;
	if ( s->type != b2_polygonShape )
		return 0;
	out[0] = (float)s->polygon.count;
	out[1] = s->polygon.radius;
	out[2] = s->polygon.centroid.x;
	out[3] = s->polygon.centroid.y;
	for ( int i = 0; i < 8; ++i )
	{
		out[4 + 2 * i] = s->polygon.vertices[i].x;
		out[5 + 2 * i] = s->polygon.vertices[i].y;
		out[20 + 2 * i] = s->polygon.normals[i].x;
		out[21 + 2 * i] = s->polygon.normals[i].y;
	}
	return s->polygon.count;
}

// colour occupancy (contacts per colour, 12 entries) from b2World_GetCounters
void ref_get_color_counts( int w, int* out )
{
	b2Counters c = b2World_GetCounters( s_worlds[w] );
	for ( int i = 0; i < 24 && i < B2_GRAPH_COLOR_COUNT; ++i )
		out[i] = c.colorCounts[i];
}

int ref_awake_body_count( int w )
{
	return b2World_GetAwakeBodyCount( s_worlds[w] );
}

// b2Body_SetAwake / b2World_EnableSleeping
void ref_body_set_awake( int w, int body, int awake )
{
	b2Body_SetAwake( ref_body_id( w, body ), awake != 0 );
}

void ref_world_enable_sleeping( int w, int enabled )
{
	b2World_EnableSleeping( s_worlds[w], enabled != 0 );
}

// Sleep-related: island id per body
int ref_body_island( int w, int body )
{
	b2World* world = ref_world( w );
	return world->bodies.data[body].islandId;
}

// Contact begin/end/hit event counts of the last step
void ref_event_counts( int w, int* out )
{
	b2ContactEvents e = b2World_GetContactEvents( s_worlds[w] );
	out[0] = e.beginCount;
	out[1] = e.endCount;
	out[2] = e.hitCount;
	b2BodyEvents be = b2World_GetBodyEvents( s_worlds[w] );
	out[3] = be.moveCount;
}

// Contact begin events (shape ids 0-based) of the last step, in event order
int ref_get_begin_events( int w, int* pairs, int cap )
{
	b2ContactEvents e = b2World_GetContactEvents( s_worlds[w] );
	int n = e.beginCount < cap ? e.beginCount : cap;
	for ( int i = 0; i < n; ++i )
	{
		pairs[2 * i] = e.beginEvents[i].shapeIdA.index1 - 1;
		pairs[2 * i + 1] = e.beginEvents[i].shapeIdB.index1 - 1;
	}
	return n;
}

// The begin events' manifolds (b2ContactBeginTouchEvent.manifold), 9 floats
// per event: normal, point count, per point the world point and separation
int ref_get_begin_manifolds( int w, float* out9, int cap )
{
	b2ContactEvents e = b2World_GetContactEvents( s_worlds[w] );
	int n = e.beginCount < cap ? e.beginCount : cap;
	for ( int i = 0; i < n; ++i )
	{
		const b2Manifold* m = &e.beginEvents[i].manifold;
		float* o = out9 + 9 * i;
		o[0] = m->normal.x;
		o[1] = m->normal.y;
		o[2] = (float)m->pointCount;
		for ( int k = 0; k < 2; ++k )
		{
			int on = k < m->pointCount;
			o[3 + 3 * k] = on ? m->points[k].point.x : 0.0f;
			o[4 + 3 * k] = on ? m->points[k].point.y : 0.0f;
			o[5 + 3 * k] = on ? m->points[k].separation : 0.0f;
		}
	}
	return n;
}

int ref_get_end_events( int w, int* pairs, int cap )
{
	b2ContactEvents e = b2World_GetContactEvents( s_worlds[w] );
	int n = e.endCount < cap ? e.endCount : cap;
	for ( int i = 0; i < n; ++i )
	{
		pairs[2 * i] = e.endEvents[i].shapeIdA.index1 - 1;
		pairs[2 * i + 1] = e.endEvents[i].shapeIdB.index1 - 1;
	}
	return n;
}

// Hit events: shapeA shapeB (ints) and point(2) normal(2) approachSpeed (floats)
int ref_get_hit_events( int w, int* ints, float* floats, int cap )
{
	b2ContactEvents e = b2World_GetContactEvents( s_worlds[w] );
	int n = e.hitCount < cap ? e.hitCount : cap;
	for ( int i = 0; i < n; ++i )
	{
		ints[2 * i] = e.hitEvents[i].shapeIdA.index1 - 1;
		ints[2 * i + 1] = e.hitEvents[i].shapeIdB.index1 - 1;
		floats[5 * i + 0] = e.hitEvents[i].point.x;
		floats[5 * i + 1] = e.hitEvents[i].point.y;
		floats[5 * i + 2] = e.hitEvents[i].normal.x;
		floats[5 * i + 3] = e.hitEvents[i].normal.y;
		floats[5 * i + 4] = e.hitEvents[i].approachSpeed;
	}
	return n;
}

// Body move events: bodyId (0-based), fellAsleep | transform p(2) q(2)
int ref_get_move_events( int w, int* ints, float* floats, int cap )
{
	b2BodyEvents e = b2World_GetBodyEvents( s_worlds[w] );
	int n = e.moveCount < cap ? e.moveCount : cap;
	for ( int i = 0; i < n; ++i )
	{
		ints[2 * i] = e.moveEvents[i].bodyId.index1 - 1;
		ints[2 * i + 1] = e.moveEvents[i].fellAsleep ? 1 : 0;
		floats[4 * i + 0] = e.moveEvents[i].transform.p.x;
		floats[4 * i + 1] = e.moveEvents[i].transform.p.y;
		floats[4 * i + 2] = e.moveEvents[i].transform.q.c;
		floats[4 * i + 3] = e.moveEvents[i].transform.q.s;
	}
	return n;
}

// Ray cast closest: returns 1 on hit; out: shape, point(2), normal(2), fraction
int ref_cast_ray_closest( int w, double ox, double oy, double tx, double ty, long long cat, long long mask, int* shape,
						  float* out )
{
	b2QueryFilter f = { (uint64_t)cat, (uint64_t)mask };
	b2RayResult r = b2World_CastRayClosest( s_worlds[w], ( b2Vec2 ){ (float)ox, (float)oy },
											( b2Vec2 ){ (float)tx, (float)ty }, f );
	if ( r.hit == false )
		return 0;
	*shape = r.shapeId.index1 - 1;
	out[0] = r.point.x;
	out[1] = r.point.y;
	out[2] = r.normal.x;
	out[3] = r.normal.y;
	out[4] = r.fraction;
	return 1;
}

typedef struct OverlapCtx
{
	int* out;
	int cap;
	int n;
} OverlapCtx;

static bool ref_overlap_cb( b2ShapeId id, void* ctx )
{
	OverlapCtx* c = ctx;
	if ( c->n < c->cap )
		c->out[c->n] = id.index1 - 1;
	c->n += 1;
	return true;
}

int ref_overlap_aabb( int w, double lx, double ly, double ux, double uy, long long cat, long long mask, int* out, int cap )
{
	b2QueryFilter f = { (uint64_t)cat, (uint64_t)mask };
	b2AABB box = { { (float)lx, (float)ly }, { (float)ux, (float)uy } };
	OverlapCtx c = { out, cap, 0 };
	b2World_OverlapAABB( s_worlds[w], box, f, ref_overlap_cb, &c );
	return c.n;
}

// Joint dump per joint id: colour, localIndex
int ref_joint_color( int w, int joint )
{
	b2World* world = ref_world( w );
	return world->joints.data[joint].colorIndex;
}

// ---------------------------------------------------------------------------
// Broadphase tree of one body type (0 static, 1 kinematic, 2 dynamic): the
// shape ids of its leaves in the order b2DynamicTree_Query visits them (the
// whole tree, every category), and the node pool's counters. These pin the
// restatement's tree topology and proxy ids.
// ---------------------------------------------------------------------------
typedef struct TreeOrderCtx
{
	int* out;
	int cap;
	int n;
} TreeOrderCtx;

static bool ref_tree_visit( int proxyId, uint64_t userData, void* context )
{
	(void)proxyId;
	TreeOrderCtx* c = context;
	if ( c->n < c->cap )
		c->out[c->n] = (int)userData;
	c->n += 1;
	return true;
}

int ref_tree_order( int w, int type, int* out, int cap )
{
	const b2DynamicTree* t = ref_world( w )->broadPhase.trees + type;
	TreeOrderCtx c = { out, cap, 0 };
	if ( t->root != B2_NULL_INDEX )
		b2DynamicTree_Query( t, b2DynamicTree_GetRootBounds( t ), B2_DEFAULT_MASK_BITS, ref_tree_visit, &c );
	return c.n;
}

// nodeCount, nodeCapacity, proxyCount, height, root, freeList
void ref_tree_stats( int w, int type, int* out6 )
{
	const b2DynamicTree* t = ref_world( w )->broadPhase.trees + type;
	out6[0] = t->nodeCount;
	out6[1] = t->nodeCapacity;
	out6[2] = t->proxyCount;
	out6[3] = b2DynamicTree_GetHeight( t );
	out6[4] = t->root;
	out6[5] = t->freeList;
}

// b2World_GetProfile of the last step (milliseconds): step, pairs, collide,
// solve, then the solver's stages in the struct's order (22 floats)
void ref_world_profile( int w, float* out22 )
{
	b2Profile p = b2World_GetProfile( s_worlds[w] );
	memcpy( out22, &p, sizeof( float ) * 22 );
}

// ---------------------------------------------------------------------------
// destroy path: b2DestroyBody, b2DestroyShape, b2DestroyJoint, b2DestroyChain
// ---------------------------------------------------------------------------
void ref_destroy_body( int w, int body )
{
	b2DestroyBody( ref_body_id( w, body ) );
}

void ref_body_set_type( int w, int body, int type )
{
	b2Body_SetType( ref_body_id( w, body ), (b2BodyType)type );
}

void ref_body_disable( int w, int body )
{
	b2Body_Disable( ref_body_id( w, body ) );
}

void ref_body_enable( int w, int body )
{
	b2Body_Enable( ref_body_id( w, body ) );
}

void ref_destroy_shape( int w, int shape, int updateBodyMass )
{
	b2World* world = ref_world( w );
	b2Shape* s = b2ShapeArray_Get( &world->shapes, shape );
	b2ShapeId id = { shape + 1, world->worldId, s->generation };
	b2DestroyShape( id, updateBodyMass != 0 );
}

void ref_destroy_joint( int w, int joint )
{
	b2World* world = ref_world( w );
	b2Joint* j = b2JointArray_Get( &world->joints, joint );
	b2JointId id = { joint + 1, world->worldId, j->generation };
	b2DestroyJoint( id );
}

void ref_destroy_chain( int w, int chain )
{
	b2World* world = ref_world( w );
	b2ChainShape* c = b2ChainShapeArray_Get( &world->chainShapes, chain );
	b2ChainId id = { chain + 1, world->worldId, c->generation };
	b2DestroyChain( id );
}

// ---------------------------------------------------------------------------
// properties: the generic get/set codes of the product's C ABI, through the
// library's own b2Body_* / b2Shape_* / b2Chain_* / b2*Joint_* calls
// ---------------------------------------------------------------------------
static b2ShapeId ref_shape_id( int w, int shape )
{
	b2World* world = ref_world( w );
	b2Shape* s = b2ShapeArray_Get( &world->shapes, shape );
	b2ShapeId id = { shape + 1, world->worldId, s->generation };
	return id;
}

static b2JointId ref_joint_id( int w, int joint )
{
	b2World* world = ref_world( w );
	b2Joint* j = b2JointArray_Get( &world->joints, joint );
	b2JointId id = { joint + 1, world->worldId, j->generation };
	return id;
}

double ref_body_get_param( int w, int body, int code )
{
	b2BodyId id = ref_body_id( w, body );
	switch ( code )
	{
		case F2D_BODY_LINEAR_DAMPING: return b2Body_GetLinearDamping( id );
		case F2D_BODY_ANGULAR_DAMPING: return b2Body_GetAngularDamping( id );
		case F2D_BODY_GRAVITY_SCALE: return b2Body_GetGravityScale( id );
		case F2D_BODY_BULLET: return b2Body_IsBullet( id );
		case F2D_BODY_FIXED_ROTATION: return b2Body_IsFixedRotation( id );
		case F2D_BODY_ENABLED: return b2Body_IsEnabled( id );
		case F2D_BODY_TYPE: return (int)b2Body_GetType( id );
		case F2D_BODY_LOCAL_CENTER_X: return b2Body_GetLocalCenterOfMass( id ).x;
		case F2D_BODY_LOCAL_CENTER_Y: return b2Body_GetLocalCenterOfMass( id ).y;
		case F2D_BODY_WORLD_CENTER_X: return b2Body_GetWorldCenterOfMass( id ).x;
		case F2D_BODY_WORLD_CENTER_Y: return b2Body_GetWorldCenterOfMass( id ).y;
		default: return 0.0;
	}
}

void ref_body_set_param( int w, int body, int code, double value )
{
	b2BodyId id = ref_body_id( w, body );
	float v = (float)value;
	switch ( code )
	{
		case F2D_BODY_LINEAR_DAMPING: b2Body_SetLinearDamping( id, v ); break;
		case F2D_BODY_ANGULAR_DAMPING: b2Body_SetAngularDamping( id, v ); break;
		case F2D_BODY_GRAVITY_SCALE: b2Body_SetGravityScale( id, v ); break;
		case F2D_BODY_BULLET: b2Body_SetBullet( id, value != 0.0 ); break;
		case F2D_BODY_FIXED_ROTATION: b2Body_SetFixedRotation( id, value != 0.0 ); break;
		default: break;
	}
}

void ref_body_set_mass_data( int w, int body, double mass, double inertia, double cx, double cy )
{
	b2MassData md = { (float)mass, { (float)cx, (float)cy }, (float)inertia };
	b2Body_SetMassData( ref_body_id( w, body ), md );
}

void ref_body_apply_mass_from_shapes( int w, int body )
{
	b2Body_ApplyMassFromShapes( ref_body_id( w, body ) );
}

double ref_shape_get_param( int w, int shape, int code )
{
	b2ShapeId id = ref_shape_id( w, shape );
	switch ( code )
	{
		case F2D_SHAPE_DENSITY: return b2Shape_GetDensity( id );
		case F2D_SHAPE_FRICTION: return b2Shape_GetFriction( id );
		case F2D_SHAPE_RESTITUTION: return b2Shape_GetRestitution( id );
		case F2D_SHAPE_SENSOR: return b2Shape_IsSensor( id );
		case F2D_SHAPE_SENSOR_EVENTS: return b2Shape_AreSensorEventsEnabled( id );
		case F2D_SHAPE_CONTACT_EVENTS: return b2Shape_AreContactEventsEnabled( id );
		case F2D_SHAPE_HIT_EVENTS: return b2Shape_AreHitEventsEnabled( id );
		case F2D_SHAPE_PRESOLVE_EVENTS: return b2Shape_ArePreSolveEventsEnabled( id );
		case F2D_SHAPE_CATEGORY: return (double)(int64_t)b2Shape_GetFilter( id ).categoryBits;
		case F2D_SHAPE_MASK: return (double)(int64_t)b2Shape_GetFilter( id ).maskBits;
		case F2D_SHAPE_GROUP: return b2Shape_GetFilter( id ).groupIndex;
		default: return 0.0;
	}
}

void ref_shape_set_param( int w, int shape, int code, double value, int flag )
{
	b2ShapeId id = ref_shape_id( w, shape );
	float v = (float)value;
	bool on = value != 0.0;
	switch ( code )
	{
		case F2D_SHAPE_DENSITY: b2Shape_SetDensity( id, v, flag != 0 ); break;
		case F2D_SHAPE_FRICTION: b2Shape_SetFriction( id, v ); break;
		case F2D_SHAPE_RESTITUTION: b2Shape_SetRestitution( id, v ); break;
		case F2D_SHAPE_SENSOR_EVENTS: b2Shape_EnableSensorEvents( id, on ); break;
		case F2D_SHAPE_CONTACT_EVENTS: b2Shape_EnableContactEvents( id, on ); break;
		case F2D_SHAPE_HIT_EVENTS: b2Shape_EnableHitEvents( id, on ); break;
		case F2D_SHAPE_PRESOLVE_EVENTS: b2Shape_EnablePreSolveEvents( id, on ); break;
		default: break;
	}
}

void ref_shape_set_filter( int w, int shape, long long categoryBits, long long maskBits, int groupIndex )
{
	b2Filter f = b2DefaultFilter();
	f.categoryBits = (uint64_t)categoryBits;
	f.maskBits = (uint64_t)maskBits;
	f.groupIndex = groupIndex;
	b2Shape_SetFilter( ref_shape_id( w, shape ), f );
}

int ref_shape_test_point( int w, int shape, double x, double y )
{
	b2Vec2 p = { (float)x, (float)y };
	return b2Shape_TestPoint( ref_shape_id( w, shape ), p );
}

void ref_chain_set_param( int w, int chain, int code, double value )
{
	b2World* world = ref_world( w );
	b2ChainShape* c = b2ChainShapeArray_Get( &world->chainShapes, chain );
	b2ChainId id = { chain + 1, world->worldId, c->generation };
	if ( code == F2D_SHAPE_FRICTION )
		b2Chain_SetFriction( id, (float)value );
	else if ( code == F2D_SHAPE_RESTITUTION )
		b2Chain_SetRestitution( id, (float)value );
}

double ref_joint_get_param( int w, int joint, int code )
{
	b2JointId id = ref_joint_id( w, joint );
	b2JointType t = b2Joint_GetType( id );
	switch ( code )
	{
		case F2D_JP_TYPE: return (int)t;
		case F2D_JP_LOCAL_ANCHOR_AX: return b2Joint_GetLocalAnchorA( id ).x;
		case F2D_JP_LOCAL_ANCHOR_AY: return b2Joint_GetLocalAnchorA( id ).y;
		case F2D_JP_LOCAL_ANCHOR_BX: return b2Joint_GetLocalAnchorB( id ).x;
		case F2D_JP_LOCAL_ANCHOR_BY: return b2Joint_GetLocalAnchorB( id ).y;
		default: break;
	}
	switch ( t )
	{
		case b2_revoluteJoint:
			switch ( code )
			{
				case F2D_JP_SPRING_ENABLED: return b2RevoluteJoint_IsSpringEnabled( id );
				case F2D_JP_SPRING_HERTZ: return b2RevoluteJoint_GetSpringHertz( id );
				case F2D_JP_SPRING_DAMPING: return b2RevoluteJoint_GetSpringDampingRatio( id );
				case F2D_JP_TARGET: return b2RevoluteJoint_GetTargetAngle( id );
				case F2D_JP_LIMIT_ENABLED: return b2RevoluteJoint_IsLimitEnabled( id );
				case F2D_JP_LOWER: return b2RevoluteJoint_GetLowerLimit( id );
				case F2D_JP_UPPER: return b2RevoluteJoint_GetUpperLimit( id );
				case F2D_JP_MOTOR_ENABLED: return b2RevoluteJoint_IsMotorEnabled( id );
				case F2D_JP_MOTOR_SPEED: return b2RevoluteJoint_GetMotorSpeed( id );
				case F2D_JP_MAX_MOTOR: return b2RevoluteJoint_GetMaxMotorTorque( id );
				case F2D_JP_MOTOR_EFFORT: return b2RevoluteJoint_GetMotorTorque( id );
				case F2D_JP_CURRENT: return b2RevoluteJoint_GetAngle( id );
			}
			break;
		case b2_prismaticJoint:
			switch ( code )
			{
				case F2D_JP_SPRING_ENABLED: return b2PrismaticJoint_IsSpringEnabled( id );
				case F2D_JP_SPRING_HERTZ: return b2PrismaticJoint_GetSpringHertz( id );
				case F2D_JP_SPRING_DAMPING: return b2PrismaticJoint_GetSpringDampingRatio( id );
				case F2D_JP_TARGET: return b2PrismaticJoint_GetTargetTranslation( id );
				case F2D_JP_LIMIT_ENABLED: return b2PrismaticJoint_IsLimitEnabled( id );
				case F2D_JP_LOWER: return b2PrismaticJoint_GetLowerLimit( id );
				case F2D_JP_UPPER: return b2PrismaticJoint_GetUpperLimit( id );
				case F2D_JP_MOTOR_ENABLED: return b2PrismaticJoint_IsMotorEnabled( id );
				case F2D_JP_MOTOR_SPEED: return b2PrismaticJoint_GetMotorSpeed( id );
				case F2D_JP_MAX_MOTOR: return b2PrismaticJoint_GetMaxMotorForce( id );
				case F2D_JP_MOTOR_EFFORT: return b2PrismaticJoint_GetMotorForce( id );
				case F2D_JP_CURRENT: return b2PrismaticJoint_GetTranslation( id );
				case F2D_JP_SPEED: return b2PrismaticJoint_GetSpeed( id );
			}
			break;
		case b2_wheelJoint:
			switch ( code )
			{
				case F2D_JP_SPRING_ENABLED: return b2WheelJoint_IsSpringEnabled( id );
				case F2D_JP_SPRING_HERTZ: return b2WheelJoint_GetSpringHertz( id );
				case F2D_JP_SPRING_DAMPING: return b2WheelJoint_GetSpringDampingRatio( id );
				case F2D_JP_LIMIT_ENABLED: return b2WheelJoint_IsLimitEnabled( id );
				case F2D_JP_LOWER: return b2WheelJoint_GetLowerLimit( id );
				case F2D_JP_UPPER: return b2WheelJoint_GetUpperLimit( id );
				case F2D_JP_MOTOR_ENABLED: return b2WheelJoint_IsMotorEnabled( id );
				case F2D_JP_MOTOR_SPEED: return b2WheelJoint_GetMotorSpeed( id );
				case F2D_JP_MAX_MOTOR: return b2WheelJoint_GetMaxMotorTorque( id );
				case F2D_JP_MOTOR_EFFORT: return b2WheelJoint_GetMotorTorque( id );
			}
			break;
		case b2_distanceJoint:
			switch ( code )
			{
				case F2D_JP_SPRING_ENABLED: return b2DistanceJoint_IsSpringEnabled( id );
				case F2D_JP_SPRING_HERTZ: return b2DistanceJoint_GetSpringHertz( id );
				case F2D_JP_SPRING_DAMPING: return b2DistanceJoint_GetSpringDampingRatio( id );
				case F2D_JP_LIMIT_ENABLED: return b2DistanceJoint_IsLimitEnabled( id );
				case F2D_JP_MOTOR_ENABLED: return b2DistanceJoint_IsMotorEnabled( id );
				case F2D_JP_MOTOR_SPEED: return b2DistanceJoint_GetMotorSpeed( id );
				case F2D_JP_MAX_MOTOR: return b2DistanceJoint_GetMaxMotorForce( id );
				case F2D_JP_MOTOR_EFFORT: return b2DistanceJoint_GetMotorForce( id );
				case F2D_JP_LENGTH: return b2DistanceJoint_GetLength( id );
				case F2D_JP_MIN_LENGTH: return b2DistanceJoint_GetMinLength( id );
				case F2D_JP_MAX_LENGTH: return b2DistanceJoint_GetMaxLength( id );
				case F2D_JP_CURRENT: return b2DistanceJoint_GetCurrentLength( id );
			}
			break;
		case b2_weldJoint:
			switch ( code )
			{
				case F2D_JP_LINEAR_HERTZ: return b2WeldJoint_GetLinearHertz( id );
				case F2D_JP_LINEAR_DAMPING: return b2WeldJoint_GetLinearDampingRatio( id );
				case F2D_JP_ANGULAR_HERTZ: return b2WeldJoint_GetAngularHertz( id );
				case F2D_JP_ANGULAR_DAMPING: return b2WeldJoint_GetAngularDampingRatio( id );
			}
			break;
		case b2_motorJoint:
			switch ( code )
			{
				case F2D_JP_LINEAR_OFFSET_X: return b2MotorJoint_GetLinearOffset( id ).x;
				case F2D_JP_LINEAR_OFFSET_Y: return b2MotorJoint_GetLinearOffset( id ).y;
				case F2D_JP_ANGULAR_OFFSET: return b2MotorJoint_GetAngularOffset( id );
				case F2D_JP_MAX_FORCE: return b2MotorJoint_GetMaxForce( id );
				case F2D_JP_MAX_TORQUE: return b2MotorJoint_GetMaxTorque( id );
				case F2D_JP_CORRECTION: return b2MotorJoint_GetCorrectionFactor( id );
			}
			break;
		case b2_mouseJoint:
			switch ( code )
			{
				case F2D_JP_TARGET_X: return b2MouseJoint_GetTarget( id ).x;
				case F2D_JP_TARGET_Y: return b2MouseJoint_GetTarget( id ).y;
				case F2D_JP_SPRING_HERTZ: return b2MouseJoint_GetSpringHertz( id );
				case F2D_JP_SPRING_DAMPING: return b2MouseJoint_GetSpringDampingRatio( id );
				case F2D_JP_MAX_FORCE: return b2MouseJoint_GetMaxForce( id );
			}
			break;
		default:
			break;
	}
	return 0.0;
}

void ref_joint_set_param( int w, int joint, int code, double value, double value2 )
{
	b2JointId id = ref_joint_id( w, joint );
	b2JointType t = b2Joint_GetType( id );
	float v = (float)value, v2 = (float)value2;
	bool on = value != 0.0;
	switch ( t )
	{
		case b2_revoluteJoint:
			switch ( code )
			{
				case F2D_JP_SPRING_ENABLED: b2RevoluteJoint_EnableSpring( id, on ); break;
				case F2D_JP_SPRING_HERTZ: b2RevoluteJoint_SetSpringHertz( id, v ); break;
				case F2D_JP_SPRING_DAMPING: b2RevoluteJoint_SetSpringDampingRatio( id, v ); break;
				case F2D_JP_TARGET: b2RevoluteJoint_SetTargetAngle( id, v ); break;
				case F2D_JP_LIMIT_ENABLED: b2RevoluteJoint_EnableLimit( id, on ); break;
				case F2D_JP_LOWER: b2RevoluteJoint_SetLimits( id, v, v2 ); break;
				case F2D_JP_MOTOR_ENABLED: b2RevoluteJoint_EnableMotor( id, on ); break;
				case F2D_JP_MOTOR_SPEED: b2RevoluteJoint_SetMotorSpeed( id, v ); break;
				case F2D_JP_MAX_MOTOR: b2RevoluteJoint_SetMaxMotorTorque( id, v ); break;
			}
			break;
		case b2_prismaticJoint:
			switch ( code )
			{
				case F2D_JP_SPRING_ENABLED: b2PrismaticJoint_EnableSpring( id, on ); break;
				case F2D_JP_SPRING_HERTZ: b2PrismaticJoint_SetSpringHertz( id, v ); break;
				case F2D_JP_SPRING_DAMPING: b2PrismaticJoint_SetSpringDampingRatio( id, v ); break;
				case F2D_JP_TARGET: b2PrismaticJoint_SetTargetTranslation( id, v ); break;
				case F2D_JP_LIMIT_ENABLED: b2PrismaticJoint_EnableLimit( id, on ); break;
				case F2D_JP_LOWER: b2PrismaticJoint_SetLimits( id, v, v2 ); break;
				case F2D_JP_MOTOR_ENABLED: b2PrismaticJoint_EnableMotor( id, on ); break;
				case F2D_JP_MOTOR_SPEED: b2PrismaticJoint_SetMotorSpeed( id, v ); break;
				case F2D_JP_MAX_MOTOR: b2PrismaticJoint_SetMaxMotorForce( id, v ); break;
			}
			break;
		case b2_wheelJoint:
			switch ( code )
			{
				case F2D_JP_SPRING_ENABLED: b2WheelJoint_EnableSpring( id, on ); break;
				case F2D_JP_SPRING_HERTZ: b2WheelJoint_SetSpringHertz( id, v ); break;
				case F2D_JP_SPRING_DAMPING: b2WheelJoint_SetSpringDampingRatio( id, v ); break;
				case F2D_JP_LIMIT_ENABLED: b2WheelJoint_EnableLimit( id, on ); break;
				case F2D_JP_LOWER: b2WheelJoint_SetLimits( id, v, v2 ); break;
				case F2D_JP_MOTOR_ENABLED: b2WheelJoint_EnableMotor( id, on ); break;
				case F2D_JP_MOTOR_SPEED: b2WheelJoint_SetMotorSpeed( id, v ); break;
				case F2D_JP_MAX_MOTOR: b2WheelJoint_SetMaxMotorTorque( id, v ); break;
			}
			break;
		case b2_distanceJoint:
			switch ( code )
			{
				case F2D_JP_SPRING_ENABLED: b2DistanceJoint_EnableSpring( id, on ); break;
				case F2D_JP_SPRING_HERTZ: b2DistanceJoint_SetSpringHertz( id, v ); break;
				case F2D_JP_SPRING_DAMPING: b2DistanceJoint_SetSpringDampingRatio( id, v ); break;
				case F2D_JP_LIMIT_ENABLED: b2DistanceJoint_EnableLimit( id, on ); break;
				case F2D_JP_MOTOR_ENABLED: b2DistanceJoint_EnableMotor( id, on ); break;
				case F2D_JP_MOTOR_SPEED: b2DistanceJoint_SetMotorSpeed( id, v ); break;
				case F2D_JP_MAX_MOTOR: b2DistanceJoint_SetMaxMotorForce( id, v ); break;
				case F2D_JP_LENGTH: b2DistanceJoint_SetLength( id, v ); break;
				case F2D_JP_MIN_LENGTH: b2DistanceJoint_SetLengthRange( id, v, v2 ); break;
			}
			break;
		case b2_weldJoint:
			switch ( code )
			{
				case F2D_JP_LINEAR_HERTZ: b2WeldJoint_SetLinearHertz( id, v ); break;
				case F2D_JP_LINEAR_DAMPING: b2WeldJoint_SetLinearDampingRatio( id, v ); break;
				case F2D_JP_ANGULAR_HERTZ: b2WeldJoint_SetAngularHertz( id, v ); break;
				case F2D_JP_ANGULAR_DAMPING: b2WeldJoint_SetAngularDampingRatio( id, v ); break;
			}
			break;
		case b2_motorJoint:
			switch ( code )
			{
				case F2D_JP_LINEAR_OFFSET_X: b2MotorJoint_SetLinearOffset( id, ( b2Vec2 ){ v, v2 } ); break;
				case F2D_JP_ANGULAR_OFFSET: b2MotorJoint_SetAngularOffset( id, v ); break;
				case F2D_JP_MAX_FORCE: b2MotorJoint_SetMaxForce( id, v ); break;
				case F2D_JP_MAX_TORQUE: b2MotorJoint_SetMaxTorque( id, v ); break;
				case F2D_JP_CORRECTION: b2MotorJoint_SetCorrectionFactor( id, v ); break;
			}
			break;
		case b2_mouseJoint:
			switch ( code )
			{
				case F2D_JP_SPRING_HERTZ: b2MouseJoint_SetSpringHertz( id, v ); break;
				case F2D_JP_SPRING_DAMPING: b2MouseJoint_SetSpringDampingRatio( id, v ); break;
				case F2D_JP_MAX_FORCE: b2MouseJoint_SetMaxForce( id, v ); break;
			}
			break;
		default:
			break;
	}
}
