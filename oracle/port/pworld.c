// World, creation path, broadphase pairs, narrowphase update, contact state
// changes and constraint-graph colouring of the restatement. TEST
// INFRASTRUCTURE (oracle). Reference files (packages/forge2d/third_party/
// box2d/src/): world.c, body.c, shape.c, broad_phase.c, contact.c,
// constraint_graph.c, id_pool.c.
//
// Contact creation order. The reference creates new contacts in broadphase
// move-array order x tree order (broad_phase.c:311-474); this port keeps the
// reference's trees operation by operation (ptree.c), so its contacts are
// created in the reference's order and take the reference's ids. A parity
// mode (orc_set_contact_plan) remains, in which the caller dictates the
// contact id of each pair created in the next step.
#include "port.h"

#include <stdlib.h>
#include <string.h>
#include <time.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define MAX_WORLDS 64
static World s_worlds[MAX_WORLDS];

void p_solve( World* w, float dt, int subSteps ); // psolver.c

static void* grow( void* p, int* cap, int need, size_t elem )
{
	if ( need <= *cap )
		return p;
	int nc = *cap < 16 ? 16 : *cap;
	while ( nc < need )
		nc *= 2;
	void* q = realloc( p, (size_t)nc * elem );
	memset( (char*)q + (size_t)( *cap ) * elem, 0, (size_t)( nc - *cap ) * elem );
	*cap = nc;
	return q;
}

World* p_world( int w )
{
	if ( w < 0 || w >= MAX_WORLDS || s_worlds[w].used == 0 )
		return NULL;
	return s_worlds + w;
}

// ---------------------------------------------------------------------------
// pair set (table.c: open addressing keyed by B2_SHAPE_PAIR_KEY)
// ---------------------------------------------------------------------------
static uint64_t pair_key( int a, int b )
{
	return a < b ? ( (uint64_t)a << 32 ) | (uint64_t)b : ( (uint64_t)b << 32 ) | (uint64_t)a;
}

static uint32_t hash64( uint64_t k )
{
	k ^= k >> 33;
	k *= 0xff51afd7ed558ccdULL;
	k ^= k >> 33;
	k *= 0xc4ceb9fe1a85ec53ULL;
	k ^= k >> 33;
	return (uint32_t)k;
}

static void pairset_rehash( PairSet* s, int ncap );

static void pairset_add( PairSet* s, uint64_t key )
{
	if ( ( s->count + 1 ) * 2 > s->cap )
		pairset_rehash( s, s->cap < 64 ? 128 : s->cap * 2 );
	uint32_t m = (uint32_t)s->cap - 1;
	uint32_t i = hash64( key ) & m;
	while ( s->keys[i] != 0 )
	{
		if ( s->keys[i] == key + 1 )
			return;
		i = ( i + 1 ) & m;
	}
	s->keys[i] = key + 1;
	s->count += 1;
}

static int pairset_contains( const PairSet* s, uint64_t key )
{
	if ( s->cap == 0 )
		return 0;
	uint32_t m = (uint32_t)s->cap - 1;
	uint32_t i = hash64( key ) & m;
	while ( s->keys[i] != 0 )
	{
		if ( s->keys[i] == key + 1 )
			return 1;
		i = ( i + 1 ) & m;
	}
	return 0;
}

static void pairset_remove( PairSet* s, uint64_t key )
{
	if ( s->cap == 0 )
		return;
	uint32_t m = (uint32_t)s->cap - 1;
	uint32_t i = hash64( key ) & m;
	while ( s->keys[i] != 0 )
	{
		if ( s->keys[i] == key + 1 )
			break;
		i = ( i + 1 ) & m;
	}
	if ( s->keys[i] == 0 )
		return;
	s->keys[i] = 0;
	s->count -= 1;
	// backward-shift deletion
	uint32_t j = i;
	while ( 1 )
	{
		j = ( j + 1 ) & m;
		if ( s->keys[j] == 0 )
			break;
		uint32_t home = hash64( s->keys[j] - 1 ) & m;
		int moveIt = ( i <= j ) ? ( home <= i || home > j ) : ( home <= i && home > j );
		if ( moveIt )
		{
			s->keys[i] = s->keys[j];
			s->keys[j] = 0;
			i = j;
		}
	}
}

static void pairset_rehash( PairSet* s, int ncap )
{
	uint64_t* old = s->keys;
	int oc = s->cap;
	s->keys = calloc( (size_t)ncap, sizeof( uint64_t ) );
	s->cap = ncap;
	s->count = 0;
	for ( int i = 0; i < oc; ++i )
		if ( old[i] )
			pairset_add( s, old[i] - 1 );
	free( old );
}

// ---------------------------------------------------------------------------
// world lifecycle (world.c:100-340)
// ---------------------------------------------------------------------------
int orc_create_world( const f2d_world_def* d, int workerCount )
{
	(void)workerCount;
	int slot = -1;
	for ( int i = 0; i < MAX_WORLDS; ++i )
		if ( s_worlds[i].used == 0 )
		{
			slot = i;
			break;
		}
	if ( slot < 0 )
		return -1;
	World* w = s_worlds + slot;
	memset( w, 0, sizeof( *w ) );
	w->used = 1;
	w->def = *d;
	w->gravity = V( (float)d->gravityX, (float)d->gravityY );
	w->restitutionThreshold = (float)d->restitutionThreshold;
	w->hitEventThreshold = (float)d->hitEventThreshold;
	w->contactHertz = (float)d->contactHertz;
	w->contactDampingRatio = (float)d->contactDampingRatio;
	w->maxContactPushSpeed = (float)d->maxContactPushSpeed;
	w->maximumLinearSpeed = (float)d->maximumLinearSpeed;
	w->enableSleep = d->enableSleep != 0;
	w->enableContinuous = d->enableContinuous != 0;
	w->enableWarmStarting = 1;
	for ( int i = 0; i < 3; ++i )
		rt_init( w->trees + i );
	p_sets_init( w );
	return slot;
}

void orc_destroy_world( int wi )
{
	World* w = p_world( wi );
	if ( w == NULL )
		return;
	free( w->bodies );
	free( w->bodyFree );
	free( w->shapes );
	free( w->shapeFree );
	free( w->contacts );
	free( w->contactFree );
	free( w->joints );
	free( w->jointFree );
	for ( int i = 0; i < w->chainCount; ++i )
		free( w->chains[i].shapeIds );
	free( w->chains );
	free( w->chainFree );
	for ( int i = 0; i < w->sensorCount; ++i )
	{
		ia_free( &w->sensors[i].overlaps1 );
		ia_free( &w->sensors[i].overlaps2 );
	}
	free( w->sensors );
	ia_free( &w->sensorBegin );
	ia_free( &w->sensorEnd );
	for ( int i = 0; i < 3; ++i )
		rt_release_all( w->trees + i );
	free( w->pairs.keys );
	free( w->moveArray );
	free( w->movedFlag );
	free( w->overflowContacts );
	free( w->overflowJoints );
	free( w->plan );
	free( w->constraints );
	free( w->beginEvents );
	ia_free( &w->pendingEnd );
	ia_free( &w->pendingSensorEnd );
	free( w->beginManifolds );
	free( w->endEvents );
	free( w->hitShapes );
	free( w->hitData );
	free( w->moveEventBodies );
	free( w->moveEventXf );
	free( w->constraintOrder );
	free( w->staticOrder );
	free( w->jointOrder );
	p_sets_free( w );
	memset( w, 0, sizeof( *w ) );
}

// The static tree's leaves in its depth-first visiting order (categories of
// zero never visited), rebuilt after the tree changed. Continuous collision
// walks this list with its box test: a query visits the overlapping leaves
// in exactly this relative order (dynamic_tree.c:1114-1170).
static int static_visit( int proxyId, int shape, void* context )
{
	(void)proxyId;
	World* w = context;
	w->staticOrder = grow( w->staticOrder, &w->staticOrderCap, w->staticOrderCount + 1, sizeof( int ) );
	w->staticOrder[w->staticOrderCount++] = shape;
	return 1;
}

void p_static_order( World* w )
{
	if ( w->staticOrderDirty == 0 )
		return;
	w->staticOrderDirty = 0;
	w->staticOrderCount = 0;
	const RTree* t = w->trees + BODY_STATIC;
	if ( t->root != P_NULL )
		rt_query( t, t->nodes[t->root].aabb, ~0ull, static_visit, w );
}

// id_pool.c:19-38: LIFO free list
static int alloc_id( int** freeList, int* freeCount, int* count )
{
	if ( *freeCount > 0 )
	{
		*freeCount -= 1;
		return ( *freeList )[*freeCount];
	}
	int id = *count;
	*count += 1;
	return id;
}

// ---------------------------------------------------------------------------
// bodies (body.c:177-330, :528-632)
// ---------------------------------------------------------------------------
int orc_create_body( int wi, const f2d_body_def* d )
{
	World* w = p_world( wi );
	int cap = w->bodyCap;
	int id = alloc_id( &w->bodyFree, &w->bodyFreeCount, &w->bodyCount );
	w->bodies = grow( w->bodies, &cap, w->bodyCount, sizeof( Body ) );
	w->bodyCap = cap;
	Body* b = w->bodies + id;
	int gen = b->generation;
	memset( b, 0, sizeof( *b ) );
	b->generation = gen + 1;
	b->used = 1;
	b->type = d->type;
	b->enabled = d->isEnabled != 0;
	b->xf.p = V( (float)d->positionX, (float)d->positionY );
	b->xf.q.c = (float)d->rotationCos;
	b->xf.q.s = (float)d->rotationSin;
	b->center = b->xf.p;
	b->rotation0 = b->xf.q;
	b->center0 = b->center;
	b->minExtent = P_HUGE;
	b->maxExtent = 0.0f;
	b->linearDamping = (float)d->linearDamping;
	b->angularDamping = (float)d->angularDamping;
	b->gravityScale = (float)d->gravityScale;
	b->sub = w->subCount > 0 ? w->subCount - 1 : 0;
	b->gravity = w->subCount > 0 ? w->subGravity : w->gravity;
	b->isBullet = d->isBullet != 0;
	b->allowFastRotation = d->allowFastRotation != 0;
	b->fixedRotation = d->fixedRotation != 0;
	if ( b->type != BODY_STATIC )
	{
		b->v = V( (float)d->linearVelocityX, (float)d->linearVelocityY );
		b->w = (float)d->angularVelocity;
	}
	b->dq.c = 1.0f;
	b->dq.s = 0.0f;
	b->headShape = P_NULL;
	b->headChain = P_NULL;
	b->headJoint = P_NULL;
	b->sleepThreshold = (float)d->sleepThreshold;
	b->enableSleep = d->enableSleep != 0;
	b->islandId = b->islandPrev = b->islandNext = P_NULL;
	b->headContactKey = P_NULL;
	b->moveEventIndex = P_NULL;
	// solver set (body.c:225-260): disabled, static, awake, or a new sleeping
	// set; dynamic and kinematic bodies get an island
	int setId;
	if ( b->enabled == 0 )
		setId = SET_DISABLED;
	else if ( b->type == BODY_STATIC )
		setId = SET_STATIC;
	else if ( d->isAwake )
		setId = SET_AWAKE;
	else
		setId = p_new_sleeping_set( w );
	p_set_body_add( w, setId, id );
	if ( setId >= SET_AWAKE )
		p_create_island_for_body( w, setId, id );
	return id;
}

static void update_mass( World* w, Body* b )
{
	b->mass = 0.0f;
	b->inertia = 0.0f;
	b->invMass = 0.0f;
	b->invInertia = 0.0f;
	b->localCenter = V( 0.0f, 0.0f );
	b->minExtent = P_HUGE;
	b->maxExtent = 0.0f;
	if ( b->type != BODY_DYNAMIC )
	{
		b->center = b->xf.p;
		if ( b->type == BODY_KINEMATIC )
		{
			for ( int s = b->headShape; s != P_NULL; s = w->shapes[s].nextShape )
			{
				float mn, mx;
				p_shape_extent( w->shapes + s, V( 0.0f, 0.0f ), &mn, &mx );
				b->minExtent = fminp( b->minExtent, mn );
				b->maxExtent = fmaxp( b->maxExtent, mx );
			}
		}
		return;
	}
	v2 localCenter = V( 0.0f, 0.0f );
	for ( int s = b->headShape; s != P_NULL; s = w->shapes[s].nextShape )
	{
		const Shape* sh = w->shapes + s;
		if ( sh->density == 0.0f )
			continue;
		MassData md = p_shape_mass( sh );
		b->mass += md.mass;
		localCenter = mulAdd( localCenter, md.mass, md.center );
		b->inertia += md.rotationalInertia;
	}
	if ( b->mass > 0.0f )
	{
		b->invMass = 1.0f / b->mass;
		localCenter = mulSV( b->invMass, localCenter );
	}
	if ( b->inertia > 0.0f && b->fixedRotation == 0 )
	{
		b->inertia -= b->mass * dot( localCenter, localCenter );
		b->invInertia = 1.0f / b->inertia;
	}
	else
	{
		b->inertia = 0.0f;
		b->invInertia = 0.0f;
	}
	v2 oldCenter = b->center;
	b->localCenter = localCenter;
	b->center = xfPoint( b->xf, b->localCenter );
	b->center0 = b->center;
	// body.c:600-606: awake bodies carry velocity at the new centre
	v2 deltaLinear = crossSV( b->w, sub( b->center, oldCenter ) );
	b->v = add( b->v, deltaLinear );
	for ( int s = b->headShape; s != P_NULL; s = w->shapes[s].nextShape )
	{
		float mn, mx;
		p_shape_extent( w->shapes + s, localCenter, &mn, &mx );
		b->minExtent = fminp( b->minExtent, mn );
		b->maxExtent = fmaxp( b->maxExtent, mx );
	}
}

// ---------------------------------------------------------------------------
// shapes (shape.c:36-180, :901-925)
// ---------------------------------------------------------------------------
static void push_move( World* w, int shapeId )
{
	Shape* s = w->shapes + shapeId;
	if ( s->moved )
		return;
	s->moved = 1;
	w->movedFlag = grow( w->movedFlag, &w->movedFlagCap, w->shapeCount + 1, 1 );
	w->movedFlag[shapeId] = 1;
	w->moveArray = grow( w->moveArray, &w->moveCap, w->moveCount + 1, sizeof( int ) );
	w->moveArray[w->moveCount++] = shapeId;
}

static int create_shape( World* w, int bodyId, const f2d_shape_def* d, const Geometry* g )
{
	int cap = w->shapeCap;
	int id = alloc_id( &w->shapeFree, &w->shapeFreeCount, &w->shapeCount );
	w->shapes = grow( w->shapes, &cap, w->shapeCount, sizeof( Shape ) );
	w->shapeCap = cap;
	Body* b = w->bodies + bodyId;
	Shape* s = w->shapes + id;
	int gen = s->generation;
	memset( s, 0, sizeof( *s ) );
	s->generation = gen + 1;
	s->used = 1;
	s->bodyId = bodyId;
	s->sub = w->bodies[bodyId].sub;
	s->g = *g;
	s->density = (float)d->density;
	s->friction = (float)d->friction;
	s->restitution = (float)d->restitution;
	s->rollingResistance = (float)d->rollingResistance;
	s->tangentSpeed = (float)d->tangentSpeed;
	s->userMaterialId = d->userMaterialId;
	s->categoryBits = (uint64_t)d->categoryBits;
	s->maskBits = (uint64_t)d->maskBits;
	s->groupIndex = d->groupIndex;
	s->isSensor = d->isSensor != 0;
	s->enableContactEvents = d->enableContactEvents != 0;
	s->enableHitEvents = d->enableHitEvents != 0;
	s->enableSensorEvents = d->enableSensorEvents != 0;
	s->enablePreSolveEvents = d->enablePreSolveEvents != 0;
	s->localCentroid = p_shape_centroid( g );
	s->proxyKey = P_NULL;
	if ( b->enabled )
	{
		int proxyType = b->type;
		box2 aabb = p_shape_aabb( &s->g, b->xf );
		aabb.lo.x -= P_SPECULATIVE;
		aabb.lo.y -= P_SPECULATIVE;
		aabb.hi.x += P_SPECULATIVE;
		aabb.hi.y += P_SPECULATIVE;
		s->aabb = aabb;
		float margin = proxyType == BODY_STATIC ? P_SPECULATIVE : P_AABB_MARGIN;
		s->fatAABB.lo.x = aabb.lo.x - margin;
		s->fatAABB.lo.y = aabb.lo.y - margin;
		s->fatAABB.hi.x = aabb.hi.x + margin;
		s->fatAABB.hi.y = aabb.hi.y + margin;
		// shape.c:901-911 b2CreateShapeProxy -> broad_phase.c:91-103
		int proxyId = rt_create_proxy( w->trees + proxyType, s->fatAABB, s->categoryBits, id );
		s->proxyKey = ( proxyId << 2 ) | proxyType;
		if ( proxyType == BODY_STATIC )
			w->staticOrderDirty = 1;
		int force = d->invokeContactCreation != 0 || d->isSensor != 0;
		if ( proxyType != BODY_STATIC || force )
			push_move( w, id );
	}
	s->sensorIndex = P_NULL;
	if ( s->isSensor )
	{
		// shape.c:144-156: a sensor record per sensor shape
		int cap = w->sensorCap;
		w->sensors = grow( w->sensors, &cap, w->sensorCount + 1, sizeof( PSensor ) );
		w->sensorCap = cap;
		PSensor* sn = w->sensors + w->sensorCount;
		memset( sn, 0, sizeof( *sn ) );
		sn->shapeId = id;
		s->sensorIndex = w->sensorCount++;
	}
	if ( b->headShape != P_NULL )
		w->shapes[b->headShape].prevShape = id;
	s->prevShape = P_NULL;
	s->nextShape = b->headShape;
	b->headShape = id;
	b->shapeCount += 1;
	if ( d->updateBodyMass )
		update_mass( w, b );
	return id;
}

int orc_create_circle_shape( int wi, int body, const f2d_shape_def* d, double cx, double cy, double radius )
{
	Geometry g = { 0 };
	g.type = SHAPE_CIRCLE;
	g.c1 = V( (float)cx, (float)cy );
	g.radius = (float)radius;
	return create_shape( p_world( wi ), body, d, &g );
}

int orc_create_capsule_shape( int wi, int body, const f2d_shape_def* d, double x1, double y1, double x2, double y2,
							  double radius )
{
	Geometry g = { 0 };
	g.type = SHAPE_CAPSULE;
	g.c1 = V( (float)x1, (float)y1 );
	g.c2 = V( (float)x2, (float)y2 );
	g.radius = (float)radius;
	return create_shape( p_world( wi ), body, d, &g );
}

int orc_create_segment_shape( int wi, int body, const f2d_shape_def* d, double x1, double y1, double x2, double y2 )
{
	Geometry g = { 0 };
	g.type = SHAPE_SEGMENT;
	g.c1 = V( (float)x1, (float)y1 );
	g.c2 = V( (float)x2, (float)y2 );
	return create_shape( p_world( wi ), body, d, &g );
}

// shape.c:339-486 b2CreateChain: count >= 4 points; a loop makes count
// segments, an open chain count - 3 (the end points are ghosts only). Each
// material is six values (friction, restitution, rollingResistance,
// tangentSpeed, userMaterialId, customColor); one for all segments or one per
// point, the segment taking its leading point's. The segments use the
// default shape definition with no contact or hit events and no mass update.
int orc_create_chain( int wi, int body, const double* points, int count, const double* materials, int materialCount,
					  long long categoryBits, long long maskBits, int groupIndex, int isLoop, int enableSensorEvents )
{
	World* w = p_world( wi );
	if ( w == NULL || body < 0 || body >= w->bodyCount || count < 4 || count > 1 << 20 ||
		 ( materialCount != 1 && materialCount != count ) )
		return -1;
	int cap = w->chainCap;
	int id = alloc_id( &w->chainFree, &w->chainFreeCount, &w->chainCount );
	w->chains = grow( w->chains, &cap, w->chainCount, sizeof( PChain ) );
	w->chainCap = cap;
	PChain* ch = w->chains + id;
	int gen = ch->generation;
	memset( ch, 0, sizeof( *ch ) );
	ch->generation = gen + 1;
	ch->used = 1;
	ch->bodyId = body;
	// shape.c:369-387: chains on a body form a list, newest first
	ch->nextChain = w->bodies[body].headChain;
	w->bodies[body].headChain = id;
	ch->count = isLoop ? count : count - 3;
	ch->shapeIds = (int*)malloc( sizeof( int ) * (size_t)ch->count );
	f2d_shape_def d = { 0 };
	d.density = 1.0;
	d.categoryBits = categoryBits;
	d.maskBits = maskBits;
	d.groupIndex = groupIndex;
	d.enableSensorEvents = enableSensorEvents != 0;
	d.invokeContactCreation = 1;
	d.updateBodyMass = 0;
	v2* pts = (v2*)malloc( sizeof( v2 ) * (size_t)count );
	for ( int i = 0; i < count; ++i )
		pts[i] = V( (float)points[2 * i], (float)points[2 * i + 1] );
	for ( int k = 0; k < ch->count; ++k )
	{
		// ghost1, point1, point2, ghost2 and the material's point index
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
		Geometry g = { 0 };
		g.type = SHAPE_CHAIN_SEGMENT;
		g.g1 = pts[i0];
		g.c1 = pts[i1];
		g.c2 = pts[i2];
		g.g2 = pts[i3];
		g.chainId = id;
		ch->shapeIds[k] = create_shape( w, body, &d, &g );
	}
	free( pts );
	return id;
}

// b2Chain_GetSegments: the chain's segment shape ids in creation order
int orc_chain_get_segments( int wi, int chain, int* out, int capacity )
{
	World* w = p_world( wi );
	if ( w == NULL || chain < 0 || chain >= w->chainCount || w->chains[chain].used == 0 )
		return 0;
	const PChain* ch = w->chains + chain;
	int n = ch->count < capacity ? ch->count : capacity;
	for ( int i = 0; i < n; ++i )
		out[i] = ch->shapeIds[i];
	return ch->count;
}

int orc_create_box_shape( int wi, int body, const f2d_shape_def* d, double hx, double hy, double cx, double cy,
						  double c, double s, double radius )
{
	Geometry g = { 0 };
	g.type = SHAPE_POLYGON;
	rot q = { (float)c, (float)s };
	g.poly = p_make_offset_rounded_box( (float)hx, (float)hy, V( (float)cx, (float)cy ), q, (float)radius );
	return create_shape( p_world( wi ), body, d, &g );
}

int orc_create_polygon_shape( int wi, int body, const f2d_shape_def* d, const double* points, int count, double radius )
{
	if ( count > P_MAX_POLY )
		return -1;
	v2 pts[P_MAX_POLY], hull[P_MAX_POLY];
	for ( int i = 0; i < count; ++i )
		pts[i] = V( (float)points[2 * i], (float)points[2 * i + 1] );
	int hc = p_compute_hull( pts, count, hull );
	if ( hc == 0 )
		return -1;
	Geometry g = { 0 };
	g.type = SHAPE_POLYGON;
	g.poly = p_make_polygon( hull, hc, (float)radius );
	return create_shape( p_world( wi ), body, d, &g );
}

// ---------------------------------------------------------------------------
// revolute joints (joint.c:146-330 b2CreateJoint, :~560 b2CreateRevoluteJoint;
// constraint_graph.c:214-288 b2AssignJointColor / b2CreateJointInGraph)
// ---------------------------------------------------------------------------
static int assign_joint_color( World* w, int ia, int ib )
{
	Body* a = w->bodies + ia;
	Body* b = w->bodies + ib;
	int staticA = a->type == BODY_STATIC;
	int staticB = b->type == BODY_STATIC;
	// unlike contacts, joints against a static body may take colour 0
	for ( int i = 0; i < P_OVERFLOW; ++i )
	{
		uint16_t bit = (uint16_t)( 1u << i );
		if ( ( staticA == 0 && ( a->colorMask & bit ) ) || ( staticB == 0 && ( b->colorMask & bit ) ) )
			continue;
		if ( staticA == 0 )
			a->colorMask |= bit;
		if ( staticB == 0 )
			b->colorMask |= bit;
		return i;
	}
	return P_OVERFLOW;
}

// joint.c:146-330 b2CreateJointInternal: id, body joint lists (new joint at
// the head), then the type's fields (set by the caller), then
// joint_finish: solver set, graph colour and island edge.
static int joint_create_common( World* w, int bodyA, int bodyB, int collideConnected, int type )
{
	int cap = w->jointCap;
	int id = alloc_id( &w->jointFree, &w->jointFreeCount, &w->jointCount );
	w->joints = grow( w->joints, &cap, w->jointCount, sizeof( Joint ) );
	w->jointCap = cap;
	Joint* j = w->joints + id;
	int gen = j->generation;
	memset( j, 0, sizeof( *j ) );
	j->generation = gen + 1;
	j->used = 1;
	j->type = type;
	j->bodyA = bodyA;
	j->bodyB = bodyB;
	j->collideConnected = collideConnected != 0;
	j->color = P_NULL;
	j->overflowIndex = P_NULL;
	Body* a = w->bodies + bodyA;
	Body* b = w->bodies + bodyB;
	j->prevA = P_NULL;
	j->nextA = a->headJoint;
	if ( a->headJoint != P_NULL )
	{
		Joint* h = w->joints + ( a->headJoint >> 1 );
		if ( a->headJoint & 1 )
			h->prevB = id << 1;
		else
			h->prevA = id << 1;
	}
	a->headJoint = id << 1;
	a->jointCount += 1;
	j->prevB = P_NULL;
	j->nextB = b->headJoint;
	if ( b->headJoint != P_NULL )
	{
		Joint* h = w->joints + ( b->headJoint >> 1 );
		if ( b->headJoint & 1 )
			h->prevB = ( id << 1 ) | 1;
		else
			h->prevA = ( id << 1 ) | 1;
	}
	b->headJoint = ( id << 1 ) | 1;
	b->jointCount += 1;
	j->constraintHertz = 60.0f;
	j->constraintDampingRatio = 2.0f;
	j->constraintSoftness.biasRate = 0.0f;
	j->constraintSoftness.massScale = 1.0f;
	j->constraintSoftness.impulseScale = 0.0f;
	return id;
}

// solver set of the joint (joint.c:196-292): disabled, static, awake (in the
// graph, waking the other body's set), or the sleeping set of its bodies;
// then the island edge (joint.c:300-306)
static void joint_finish( World* w, int id )
{
	Joint* j = w->joints + id;
	Body* a = w->bodies + j->bodyA;
	Body* b = w->bodies + j->bodyB;
	j->islandId = j->islandPrev = j->islandNext = P_NULL;
	int setA = a->setIndex, setB = b->setIndex;
	int maxSet = setA > setB ? setA : setB;
	if ( setA == SET_DISABLED || setB == SET_DISABLED )
		j->setIndex = SET_DISABLED;
	else if ( setA == SET_STATIC && setB == SET_STATIC )
		j->setIndex = SET_STATIC;
	else if ( setA == SET_AWAKE || setB == SET_AWAKE )
	{
		if ( maxSet >= SET_FIRST_SLEEPING )
			p_wake_solver_set( w, maxSet );
		j->setIndex = SET_AWAKE;
		p_add_joint_to_graph( w, id );
	}
	else
	{
		j->setIndex = maxSet;
		p_set_joint_add( w, maxSet, id );
		if ( setA != setB && setA >= SET_FIRST_SLEEPING && setB >= SET_FIRST_SLEEPING )
			p_merge_solver_sets( w, setA, setB );
	}
	if ( w->joints[id].setIndex > SET_DISABLED )
		p_link_joint( w, id, 1 );
}

int orc_create_revolute_joint( int wi, const f2d_revolute_def* d )
{
	World* w = p_world( wi );
	if ( w == NULL || d->bodyA < 0 || d->bodyA >= w->bodyCount || d->bodyB < 0 || d->bodyB >= w->bodyCount )
		return -1;
	int id = joint_create_common( w, d->bodyA, d->bodyB, d->collideConnected, P_JOINT_REVOLUTE );
	Joint* j = w->joints + id;
	j->localOriginAnchorA = V( (float)d->localAnchorAX, (float)d->localAnchorAY );
	j->localOriginAnchorB = V( (float)d->localAnchorBX, (float)d->localAnchorBY );
	j->referenceAngle = fclampp( (float)d->referenceAngle, -P_PI, P_PI );
	j->targetAngle = fclampp( (float)d->targetAngle, -P_PI, P_PI );
	j->hertz = (float)d->hertz;
	j->dampingRatio = (float)d->dampingRatio;
	j->lowerAngle = (float)d->lowerAngle;
	j->upperAngle = (float)d->upperAngle;
	j->maxMotorTorque = (float)d->maxMotorTorque;
	j->motorSpeed = (float)d->motorSpeed;
	j->enableSpring = d->enableSpring != 0;
	j->enableLimit = d->enableLimit != 0;
	j->enableMotor = d->enableMotor != 0;
	j->drawSize = (float)d->drawSize;
	joint_finish( w, id );
	// joint.c:549-553: a joint that blocks collision ends its bodies' contacts
	p_joint_created( w, id );
	return id;
}

// joint.c:609-649 b2CreateWeldJoint, :353-404 b2CreateDistanceJoint
int orc_create_joint( int wi, const f2d_joint_def* d )
{
	World* w = p_world( wi );
	if ( w == NULL || d->bodyA < 0 || d->bodyA >= w->bodyCount || d->bodyB < 0 || d->bodyB >= w->bodyCount )
		return -1;
	if ( d->type < P_JOINT_WELD || d->type > P_JOINT_FILTER )
		return -1;
	// joint.c:444-478 the mouse joint reads the bodies' transforms before the
	// joint exists; joint.c:480-502 a filter joint never lets the bodies collide
	xform xfA = w->bodies[d->bodyA].xf, xfB = w->bodies[d->bodyB].xf;
	int collide = d->type == P_JOINT_FILTER ? 0 : d->collideConnected;
	int id = joint_create_common( w, d->bodyA, d->bodyB, collide, d->type );
	Joint* j = w->joints + id;
	j->localOriginAnchorA = V( (float)d->localAnchorAX, (float)d->localAnchorAY );
	j->localOriginAnchorB = V( (float)d->localAnchorBX, (float)d->localAnchorBY );
	if ( d->type == P_JOINT_PRISMATIC || d->type == P_JOINT_WHEEL )
	{
		// joint.c:559-649
		j->localAxisA = normalize( V( (float)d->localAxisAX, (float)d->localAxisAY ) );
		j->lowerTranslation = (float)d->lowerTranslation;
		j->upperTranslation = (float)d->upperTranslation;
		j->hertz = (float)d->hertz;
		j->dampingRatio = (float)d->dampingRatio;
		j->motorSpeed = (float)d->motorSpeed;
		j->enableSpring = d->enableSpring != 0;
		j->enableLimit = d->enableLimit != 0;
		j->enableMotor = d->enableMotor != 0;
		if ( d->type == P_JOINT_PRISMATIC )
		{
			j->referenceAngle = (float)d->referenceAngle;
			j->targetTranslation = (float)d->targetTranslation;
			j->maxMotorForce = (float)d->maxMotorForce;
		}
		else
			j->maxMotorTorque = (float)d->maxMotorTorque;
	}
	else if ( d->type == P_JOINT_MOTOR )
	{
		// joint.c:406-442
		j->localOriginAnchorA = V( 0.0f, 0.0f );
		j->localOriginAnchorB = V( 0.0f, 0.0f );
		j->linearOffset = V( (float)d->linearOffsetX, (float)d->linearOffsetY );
		j->angularOffset = (float)d->angularOffset;
		j->maxForce = (float)d->maxForce;
		j->maxTorque = (float)d->maxTorque;
		j->correctionFactor = fclampp( (float)d->correctionFactor, 0.0f, 1.0f );
	}
	else if ( d->type == P_JOINT_MOUSE )
	{
		v2 target = V( (float)d->targetX, (float)d->targetY );
		j->localOriginAnchorA = invXfPoint( xfA, target );
		j->localOriginAnchorB = invXfPoint( xfB, target );
		j->targetA = target;
		j->hertz = (float)d->hertz;
		j->dampingRatio = (float)d->dampingRatio;
		j->maxForce = (float)d->maxForce;
	}
	else if ( d->type == P_JOINT_FILTER )
	{
		j->localOriginAnchorA = V( 0.0f, 0.0f );
		j->localOriginAnchorB = V( 0.0f, 0.0f );
	}
	else if ( d->type == P_JOINT_WELD )
	{
		j->referenceAngle = (float)d->referenceAngle;
		j->linearHertz = (float)d->linearHertz;
		j->linearDampingRatio = (float)d->linearDampingRatio;
		j->angularHertz = (float)d->angularHertz;
		j->angularDampingRatio = (float)d->angularDampingRatio;
	}
	else
	{
		j->length = fmaxp( (float)d->length, P_LINEAR_SLOP );
		j->hertz = (float)d->hertz;
		j->dampingRatio = (float)d->dampingRatio;
		j->minLength = fmaxp( (float)d->minLength, P_LINEAR_SLOP );
		j->maxLength = fmaxp( (float)d->minLength, (float)d->maxLength );
		j->maxMotorForce = (float)d->maxMotorForce;
		j->motorSpeed = (float)d->motorSpeed;
		j->enableSpring = d->enableSpring != 0;
		j->enableLimit = d->enableLimit != 0;
		j->enableMotor = d->enableMotor != 0;
	}
	joint_finish( w, id );
	// joint.c:396-400 (and the other constructors but the mouse and filter
	// joints): a joint that blocks collision ends its bodies' contacts
	if ( d->type != P_JOINT_MOUSE && d->type != P_JOINT_FILTER )
		p_joint_created( w, id );
	return id;
}

// revolute_joint.c:129-168, prismatic_joint.c:111-150, wheel_joint.c:100-140,
// distance_joint.c:138-175: motor setters of the motorised joint types (no
// wake; switching the motor clears its impulse). `maxMotor` is the revolute
// and wheel torque, the prismatic and distance force.
void orc_joint_set_motor( int wi, int jid, int enable, double speed, double maxMotor )
{
	World* w = p_world( wi );
	if ( w == NULL || jid < 0 || jid >= w->jointCount )
		return;
	Joint* j = w->joints + jid;
	if ( j->type != P_JOINT_REVOLUTE && j->type != P_JOINT_PRISMATIC && j->type != P_JOINT_WHEEL &&
		 j->type != P_JOINT_DISTANCE )
		return;
	if ( ( enable != 0 ) != ( j->enableMotor != 0 ) )
	{
		j->enableMotor = enable != 0;
		j->motorImpulse = 0.0f;
	}
	j->motorSpeed = (float)speed;
	if ( j->type == P_JOINT_REVOLUTE || j->type == P_JOINT_WHEEL )
		j->maxMotorTorque = (float)maxMotor;
	else
		j->maxMotorForce = (float)maxMotor;
}

// revolute_joint.c:84-127, prismatic_joint.c:68-109, wheel_joint.c:57-98:
// b2*Joint_EnableLimit then b2*Joint_SetLimits (a change clears the limit
// impulses; the bounds are stored as min, max)
void orc_joint_set_limits( int wi, int jid, int enable, double lower, double upper )
{
	World* w = p_world( wi );
	if ( w == NULL || jid < 0 || jid >= w->jointCount )
		return;
	Joint* j = w->joints + jid;
	if ( j->type != P_JOINT_REVOLUTE && j->type != P_JOINT_PRISMATIC && j->type != P_JOINT_WHEEL )
		return;
	if ( ( enable != 0 ) != ( j->enableLimit != 0 ) )
	{
		j->enableLimit = enable != 0;
		j->lowerImpulse = 0.0f;
		j->upperImpulse = 0.0f;
	}
	float lo = (float)lower, hi = (float)upper;
	float* cl = j->type == P_JOINT_REVOLUTE ? &j->lowerAngle : &j->lowerTranslation;
	float* cu = j->type == P_JOINT_REVOLUTE ? &j->upperAngle : &j->upperTranslation;
	if ( lo != *cl || hi != *cu )
	{
		*cl = fminp( lo, hi );
		*cu = fmaxp( lo, hi );
		j->lowerImpulse = 0.0f;
		j->upperImpulse = 0.0f;
	}
}

// joint.c:1061-1135 b2Joint_GetConstraintForce / GetConstraintTorque with the
// per-type b2Get*JointForce / Torque (the last step's impulses times inv_h);
// out3 = force.x, force.y, torque
void orc_joint_get_constraint( int wi, int jid, float* out3 )
{
	out3[0] = out3[1] = out3[2] = 0.0f;
	World* w = p_world( wi );
	if ( w == NULL || jid < 0 || jid >= w->jointCount )
		return;
	const Joint* j = w->joints + jid;
	float inv_h = w->inv_h;
	v2 f = V( 0.0f, 0.0f );
	float t = 0.0f;
	switch ( j->type )
	{
		case P_JOINT_REVOLUTE: // revolute_joint.c:176-187
			f = mulSV( inv_h, j->linearImpulse );
			t = inv_h * ( j->motorImpulse + j->lowerImpulse - j->upperImpulse );
			break;
		case P_JOINT_WELD: // weld_joint.c:66-75
			f = mulSV( inv_h, j->linearImpulse );
			t = inv_h * j->angularImpulse;
			break;
		case P_JOINT_MOTOR: // motor_joint.c:74-83
		case P_JOINT_MOUSE: // mouse_joint.c:66-75
			f = mulSV( inv_h, j->linearImpulse );
			t = inv_h * j->angularImpulse;
			break;
		case P_JOINT_DISTANCE: // distance_joint.c:185-198
		{
			v2 pA = xfPoint( w->bodies[j->bodyA].xf, j->localOriginAnchorA );
			v2 pB = xfPoint( w->bodies[j->bodyB].xf, j->localOriginAnchorB );
			v2 axis = normalize( sub( pB, pA ) );
			float force = ( j->impulse + j->lowerImpulse - j->upperImpulse + j->motorImpulse ) * inv_h;
			f = mulSV( force, axis );
			break;
		}
		case P_JOINT_PRISMATIC: // prismatic_joint.c:211-232
		{
			v2 axisA = rotate( w->bodies[j->bodyA].xf.q, j->localAxisA );
			v2 perpA = leftPerp( axisA );
			float perpForce = inv_h * j->prismaticImpulse.x;
			float axialForce = inv_h * ( j->motorImpulse + j->lowerImpulse - j->upperImpulse );
			f = add( mulSV( perpForce, perpA ), mulSV( axialForce, axisA ) );
			t = inv_h * j->prismaticImpulse.y;
			break;
		}
		case P_JOINT_WHEEL: // wheel_joint.c:147-165 (axis of the last step)
		{
			v2 perpA = leftPerp( j->axisA );
			float perpForce = inv_h * j->perpImpulse;
			float axialForce = inv_h * ( j->springImpulse + j->lowerImpulse - j->upperImpulse );
			f = add( mulSV( perpForce, perpA ), mulSV( axialForce, j->axisA ) );
			t = inv_h * j->motorImpulse;
			break;
		}
		default:
			break;
	}
	out3[0] = f.x;
	out3[1] = f.y;
	out3[2] = t;
}

// mouse_joint.c:14-19 b2MouseJoint_SetTarget (no wake)
void orc_mouse_joint_set_target( int wi, int jid, double x, double y )
{
	World* w = p_world( wi );
	if ( w == NULL || jid < 0 || jid >= w->jointCount || w->joints[jid].type != P_JOINT_MOUSE )
		return;
	w->joints[jid].targetA = V( (float)x, (float)y );
}

// constraint_graph.c:271-288 b2CreateJointInGraph / b2AddJointToGraph
void p_add_joint_to_graph( World* w, int jid )
{
	Joint* j = w->joints + jid;
	j->color = assign_joint_color( w, j->bodyA, j->bodyB );
	j->colorBodies = ( w->bodies[j->bodyA].type != BODY_STATIC ? 1 : 0 ) | ( w->bodies[j->bodyB].type != BODY_STATIC ? 2 : 0 );
	if ( j->color == P_OVERFLOW )
	{
		w->overflowJoints = grow( w->overflowJoints, &w->overflowJointCap, w->overflowJointCount + 1, sizeof( int ) );
		j->overflowIndex = w->overflowJointCount;
		w->overflowJoints[w->overflowJointCount++] = jid;
	}
}

// constraint_graph.c:290-318 b2RemoveJointFromGraph (swap-remove in the
// overflow array; colour bits cleared otherwise)
void p_remove_joint_from_graph( World* w, int jid )
{
	Joint* j = w->joints + jid;
	if ( j->color == P_NULL )
		return;
	if ( j->color != P_OVERFLOW )
	{
		// the bits its colouring set: the reference clears both bodies' bits
		// (constraint_graph.c:303-308), which differs only for a body that was
		// static when the joint was coloured and is not any more (a type
		// change), where it would free a bit another joint of that body holds
		uint16_t bit = (uint16_t)( 1u << j->color );
		if ( j->colorBodies & 1 )
			w->bodies[j->bodyA].colorMask &= (uint16_t)~bit;
		if ( j->colorBodies & 2 )
			w->bodies[j->bodyB].colorMask &= (uint16_t)~bit;
	}
	else
	{
		int idx = j->overflowIndex;
		int last = w->overflowJointCount - 1;
		if ( idx != last )
		{
			int moved = w->overflowJoints[last];
			w->overflowJoints[idx] = moved;
			w->joints[moved].overflowIndex = idx;
		}
		w->overflowJointCount -= 1;
		j->overflowIndex = P_NULL;
	}
	j->color = P_NULL;
}

int orc_joint_color( int wi, int joint )
{
	World* w = p_world( wi );
	if ( w == NULL || joint < 0 || joint >= w->jointCount )
		return P_NULL;
	return w->joints[joint].color;
}

// ---------------------------------------------------------------------------
// joint exclusion (body.c:1861-1897 b2ShouldBodiesCollide)
// ---------------------------------------------------------------------------
static int should_bodies_collide( World* w, int ia, int ib )
{
	Body* a = w->bodies + ia;
	Body* b = w->bodies + ib;
	if ( a->type != BODY_DYNAMIC && b->type != BODY_DYNAMIC )
		return 0;
	int key, other;
	if ( a->jointCount < b->jointCount )
	{
		key = a->headJoint;
		other = ib;
	}
	else
	{
		key = b->headJoint;
		other = ia;
	}
	while ( key != P_NULL )
	{
		int jid = key >> 1;
		int edge = key & 1;
		Joint* j = w->joints + jid;
		int otherBody = edge == 0 ? j->bodyB : j->bodyA;
		if ( j->collideConnected == 0 && otherBody == other )
			return 0;
		key = edge == 0 ? j->nextA : j->nextB;
	}
	return 1;
}

// shape.h:122-130
static int should_shapes_collide( const Shape* a, const Shape* b )
{
	if ( a->groupIndex == b->groupIndex && a->groupIndex != 0 )
		return a->groupIndex > 0;
	return ( a->maskBits & b->categoryBits ) != 0 && ( a->categoryBits & b->maskBits ) != 0;
}

// ---------------------------------------------------------------------------
// contact creation (contact.c:186-330)
// ---------------------------------------------------------------------------
static int create_contact_with_id( World* w, int shapeIdA, int shapeIdB, int id )
{
	Shape* sa = w->shapes + shapeIdA;
	Shape* sb = w->shapes + shapeIdB;
	int primary;
	if ( p_manifold_registered( sa->g.type, sb->g.type, &primary ) == 0 )
		return -1;
	if ( primary == 0 )
	{
		int t = shapeIdA;
		shapeIdA = shapeIdB;
		shapeIdB = t;
		sa = w->shapes + shapeIdA;
		sb = w->shapes + shapeIdB;
	}
	w->contacts = grow( w->contacts, &w->contactCap, id + 1, sizeof( Contact ) );
	if ( id >= w->contactCount )
	{
		// ids between the old count and id become free (parity plans may skip)
		for ( int k = w->contactCount; k < id; ++k )
		{
			w->contactFree = realloc( w->contactFree, sizeof( int ) * ( w->contactFreeCount + 1 ) );
			w->contactFree[w->contactFreeCount++] = k;
		}
		w->contactCount = id + 1;
	}
	Contact* c = w->contacts + id;
	memset( c, 0, sizeof( *c ) );
	c->used = 1;
	c->shapeA = shapeIdA;
	c->shapeB = shapeIdB;
	c->bodyA = sa->bodyId;
	c->bodyB = sb->bodyId;
	c->color = P_NULL;
	c->overflowIndex = P_NULL;
	c->enableContactEvents = ( sa->enableContactEvents || sb->enableContactEvents ) ? 1 : 0;
	// world.c:88-98 default mixing: sqrt(fA*fB), max(rA, rB)
	c->friction = sqrtf( sa->friction * sb->friction );
	c->restitution = sa->restitution > sb->restitution ? sa->restitution : sb->restitution;
	c->simFlags = 0;
	if ( sa->enablePreSolveEvents || sb->enablePreSolveEvents )
		c->simFlags |= SIM_PRESOLVE;
	// contact.c:206-215: awake set when either body is awake, else disabled
	c->setIndex = ( p_body_awake( w, c->bodyA ) || p_body_awake( w, c->bodyB ) ) ? SET_AWAKE : SET_DISABLED;
	c->islandId = c->islandPrev = c->islandNext = P_NULL;
	p_contact_edges_link( w, id );
	pairset_add( &w->pairs, pair_key( shapeIdA, shapeIdB ) );
	return id;
}

static void free_contact_id( World* w, int id )
{
	w->contactFree = realloc( w->contactFree, sizeof( int ) * ( w->contactFreeCount + 1 ) );
	w->contactFree[w->contactFreeCount++] = id;
}

static int take_contact_id( World* w, int id )
{
	// remove a specific id from the free list (parity mode)
	for ( int k = w->contactFreeCount - 1; k >= 0; --k )
	{
		if ( w->contactFree[k] == id )
		{
			memmove( w->contactFree + k, w->contactFree + k + 1, sizeof( int ) * ( w->contactFreeCount - k - 1 ) );
			w->contactFreeCount -= 1;
			return 1;
		}
	}
	return id >= w->contactCount;
}

void orc_set_contact_plan( int wi, const int* rows, int count )
{
	World* w = p_world( wi );
	w->plan = grow( w->plan, &w->planCap, 3 * count, sizeof( int ) );
	memcpy( w->plan, rows, sizeof( int ) * 3 * (size_t)count );
	w->planCount = count;
}

// ---------------------------------------------------------------------------
// broadphase pair finding (broad_phase.c:160-474 b2PairQueryCallback,
// b2FindPairsTask, b2UpdateBroadPhasePairs). Every moved proxy, in move-array
// order, queries the kinematic and static trees (dynamic proxies only) and
// then the dynamic tree; each pair the callback keeps is PREPENDED to the
// proxy's list, so a proxy's pairs come out dynamic-tree first, each tree's
// leaves left to right (the reverse of the depth-first visit). Contacts are
// created proxy by proxy in that order.
// ---------------------------------------------------------------------------
typedef struct Cand
{
	uint64_t key;
	int a, b; // ordered by proxy key: a has the smaller proxy key
} Cand;

typedef struct PairQuery
{
	World* w;
	int queryShape, queryProxyKey, treeType;
	Cand* list;
	int n, cap;
} PairQuery;

// broad_phase.c:160-266 b2PairQueryCallback (the custom filter, its last
// test, runs after the queries: see update_pairs)
static int pair_visit( int proxyId, int shape, void* context )
{
	PairQuery* q = context;
	World* w = q->w;
	int proxyKey = ( proxyId << 2 ) | q->treeType;
	if ( proxyKey == q->queryProxyKey )
		return 1;
	const unsigned char* moved = w->movedFlag;
	if ( ( q->queryProxyKey & 3 ) == BODY_DYNAMIC )
	{
		// both moving: the pair belongs to the smaller proxy key's query
		if ( q->treeType == BODY_DYNAMIC && proxyKey < q->queryProxyKey && moved[shape] )
			return 1;
	}
	else if ( moved[shape] )
		return 1;
	uint64_t key = pair_key( shape, q->queryShape );
	if ( pairset_contains( &w->pairs, key ) )
		return 1;
	int a = proxyKey < q->queryProxyKey ? shape : q->queryShape;
	int b = proxyKey < q->queryProxyKey ? q->queryShape : shape;
	Shape* sa = w->shapes + a;
	Shape* sb = w->shapes + b;
	if ( sa->bodyId == sb->bodyId )
		return 1;
	if ( sa->sensorIndex != P_NULL || sb->sensorIndex != P_NULL )
		return 1;
	if ( should_shapes_collide( sa, sb ) == 0 )
		return 1;
	if ( should_bodies_collide( w, sa->bodyId, sb->bodyId ) == 0 )
		return 1;
	// sub-worlds of the batched form never meet (each is a world of its own)
	if ( sa->sub != sb->sub )
		return 1;
	q->list = grow( q->list, &q->cap, q->n + 1, sizeof( Cand ) );
	Cand* c = q->list + q->n;
	c->key = key;
	c->a = a;
	c->b = b;
	q->n += 1;
	return 1;
}

static void update_pairs( World* w )
{
	if ( w->moveCount == 0 )
	{
		w->planCount = 0;
		return;
	}
	int nm = w->moveCount;
	int nthreads = 1;
#ifdef _OPENMP
	nthreads = omp_get_max_threads();
#endif
	// broad_phase.c:311-372: each thread takes one contiguous run of the move
	// array (schedule static), so the threads' lists concatenated in thread
	// order are the move-array order
	PairQuery* tq = calloc( (size_t)nthreads, sizeof( PairQuery ) );
#pragma omp parallel
	{
		int t = 0;
#ifdef _OPENMP
		t = omp_get_thread_num();
#endif
		PairQuery* q = tq + t;
		q->w = w;
#pragma omp for schedule( static )
		for ( int i = 0; i < nm; ++i )
		{
			int shapeId = w->moveArray[i];
			Shape* s = w->shapes + shapeId;
			if ( s->used == 0 || s->proxyKey == P_NULL )
				continue;
			int type = s->proxyKey & 3;
			const RTree* base = w->trees + type;
			box2 fat = base->nodes[s->proxyKey >> 2].aabb;
			q->queryShape = shapeId;
			q->queryProxyKey = s->proxyKey;
			int first = q->n;
			if ( type == BODY_DYNAMIC )
			{
				q->treeType = BODY_KINEMATIC;
				rt_query( w->trees + BODY_KINEMATIC, fat, ~0ull, pair_visit, q );
				q->treeType = BODY_STATIC;
				rt_query( w->trees + BODY_STATIC, fat, ~0ull, pair_visit, q );
			}
			q->treeType = BODY_DYNAMIC;
			rt_query( w->trees + BODY_DYNAMIC, fat, ~0ull, pair_visit, q );
			// prepend order: this proxy's pairs in reverse visiting order
			for ( int lo = first, hi = q->n - 1; lo < hi; ++lo, --hi )
			{
				Cand tmp = q->list[lo];
				q->list[lo] = q->list[hi];
				q->list[hi] = tmp;
			}
		}
	}
	Cand* cands = NULL;
	int nc = 0, capc = 0;
	for ( int t = 0; t < nthreads; ++t )
	{
		if ( tq[t].n > 0 )
		{
			cands = grow( cands, &capc, nc + tq[t].n, sizeof( Cand ) );
			memcpy( cands + nc, tq[t].list, sizeof( Cand ) * (size_t)tq[t].n );
			nc += tq[t].n;
		}
		free( tq[t].list );
	}
	free( tq );
	// broad_phase.c:267-278: the custom filter is the last test of a new pair
	// (A is the shape with the smaller proxy key)
	if ( w->customFilter != NULL )
	{
		int v = 0;
		for ( int i = 0; i < nc; ++i )
			if ( w->customFilter( cands[i].a, cands[i].b, w->customFilterContext ) )
				cands[v++] = cands[i];
		nc = v;
	}
	// create contacts in the reference's order or per plan. A
	// plan's contacts are created in the order the reference's id pool handed
	// their ids out (LIFO free list, then fresh ids), which is the order the
	// reference created them in; that order is visible in the bodies'
	// contact lists and, through island splits, in what sleeps and wakes.
	int* planId = (int*)malloc( sizeof( int ) * (size_t)( nc > 0 ? nc : 1 ) );
	long long* rank = (long long*)malloc( sizeof( long long ) * (size_t)( nc > 0 ? nc : 1 ) );
	int* createOrder = (int*)malloc( sizeof( int ) * (size_t)( nc > 0 ? nc : 1 ) );
	for ( int i = 0; i < nc; ++i )
	{
		planId[i] = -1;
		rank[i] = (long long)i;
		createOrder[i] = i;
		if ( w->planCount == 0 )
			continue;
		for ( int k = 0; k < w->planCount; ++k )
		{
			const int* row = w->plan + 3 * k;
			if ( pair_key( row[1], row[2] ) == cands[i].key )
			{
				planId[i] = row[0];
				break;
			}
		}
		int id = planId[i];
		long long r = 4ll * nc + 4ll * w->contactCount + i;
		for ( int k = w->contactFreeCount - 1; k >= 0 && id >= 0; --k )
			if ( w->contactFree[k] == id )
			{
				r = (long long)( w->contactFreeCount - 1 - k );
				break;
			}
		if ( id >= w->contactCount )
			r = (long long)w->contactFreeCount + ( id - w->contactCount );
		rank[i] = r;
	}
	if ( w->planCount > 0 )
	{
		// insertion sort by rank (a step creates few contacts)
		for ( int i = 1; i < nc; ++i )
		{
			int v = createOrder[i];
			int j = i - 1;
			while ( j >= 0 && rank[createOrder[j]] > rank[v] )
			{
				createOrder[j + 1] = createOrder[j];
				j -= 1;
			}
			createOrder[j + 1] = v;
		}
	}
	for ( int o = 0; o < nc; ++o )
	{
		int i = createOrder[o];
		int id = planId[i];
		if ( id >= 0 )
		{
			take_contact_id( w, id );
		}
		else
		{
			id = alloc_id( &w->contactFree, &w->contactFreeCount, &w->contactCount );
		}
		create_contact_with_id( w, cands[i].a, cands[i].b, id );
	}
	free( planId );
	free( rank );
	free( createOrder );
	// reset move buffer
	for ( int i = 0; i < w->moveCount; ++i )
	{
		w->shapes[w->moveArray[i]].moved = 0;
		w->movedFlag[w->moveArray[i]] = 0;
	}
	w->moveCount = 0;
	w->planCount = 0;
	free( cands );
}

// ---------------------------------------------------------------------------
// narrowphase update (world.c:357-445 b2CollideTask, contact.c:472-600)
// ---------------------------------------------------------------------------
static void update_contact( World* w, Contact* c )
{
	Shape* sa = w->shapes + c->shapeA;
	Shape* sb = w->shapes + c->shapeB;
	if ( boxOverlaps( sa->fatAABB, sb->fatAABB ) == 0 )
	{
		c->simFlags |= SIM_DISJOINT;
		c->simFlags &= ~SIM_TOUCHING;
		return;
	}
	int wasTouching = ( c->simFlags & SIM_TOUCHING ) != 0;
	Body* ba = w->bodies + sa->bodyId;
	Body* bb = w->bodies + sb->bodyId;
	c->invMassA = ba->invMass;
	c->invIA = ba->invInertia;
	c->invMassB = bb->invMass;
	c->invIB = bb->invInertia;
	xform xfA = ba->xf;
	xform xfB = bb->xf;
	v2 centerOffsetA = rotate( xfA.q, ba->localCenter );
	v2 centerOffsetB = rotate( xfB.q, bb->localCenter );

	Manifold old = c->m;
	c->m = p_collide( &sa->g, xfA, &sb->g, xfB, &c->cache );
	c->friction = sqrtf( sa->friction * sb->friction );
	c->restitution = sa->restitution > sb->restitution ? sa->restitution : sb->restitution;
	if ( sa->rollingResistance > 0.0f || sb->rollingResistance > 0.0f )
	{
		float ra = p_shape_radius( &sa->g );
		float rb = p_shape_radius( &sb->g );
		float mr = fmaxp( ra, rb );
		c->rollingResistance = fmaxp( sa->rollingResistance, sb->rollingResistance ) * mr;
	}
	else
		c->rollingResistance = 0.0f;
	c->tangentSpeed = sa->tangentSpeed + sb->tangentSpeed;
	int pointCount = c->m.pointCount;
	int touching = pointCount > 0;
	if ( touching && w->preSolve != NULL && ( c->simFlags & SIM_PRESOLVE ) )
	{
		// contact.c:504-517: the user may disable the contact for this step
		f2d_manifold_view mv;
		memset( &mv, 0, sizeof( mv ) );
		mv.normalX = c->m.normal.x;
		mv.normalY = c->m.normal.y;
		mv.pointCount = pointCount;
		for ( int i = 0; i < pointCount; ++i )
		{
			const ManifoldPoint* mp = c->m.points + i;
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
		touching = w->preSolve( c->shapeA, c->shapeB, &mv, w->preSolveContext ) != 0;
		if ( touching == 0 )
		{
			pointCount = 0;
			c->m.pointCount = 0;
		}
	}
	if ( touching && ( sa->enableHitEvents || sb->enableHitEvents ) )
		c->simFlags |= SIM_HIT_EVENT;
	else
		c->simFlags &= ~SIM_HIT_EVENT;
	if ( pointCount > 0 )
		c->m.rollingImpulse = old.rollingImpulse;
	for ( int i = 0; i < pointCount; ++i )
	{
		ManifoldPoint* mp2 = c->m.points + i;
		mp2->anchorA = sub( mp2->anchorA, centerOffsetA );
		mp2->anchorB = sub( mp2->anchorB, centerOffsetB );
		mp2->normalImpulse = 0.0f;
		mp2->tangentImpulse = 0.0f;
		mp2->totalNormalImpulse = 0.0f;
		mp2->normalVelocity = 0.0f;
		mp2->persisted = false;
		uint16_t id2 = mp2->id;
		for ( int j = 0; j < old.pointCount; ++j )
		{
			ManifoldPoint* mp1 = old.points + j;
			if ( mp1->id == id2 )
			{
				mp2->normalImpulse = mp1->normalImpulse;
				mp2->tangentImpulse = mp1->tangentImpulse;
				mp2->persisted = true;
				mp1->normalImpulse = 0.0f;
				mp1->tangentImpulse = 0.0f;
				break;
			}
		}
	}
	if ( touching )
		c->simFlags |= SIM_TOUCHING;
	else
		c->simFlags &= ~SIM_TOUCHING;
	if ( touching && !wasTouching )
		c->simFlags |= SIM_STARTED;
	else if ( !touching && wasTouching )
		c->simFlags |= SIM_STOPPED;
}

// ---------------------------------------------------------------------------
// constraint graph (constraint_graph.c:68-212)
// ---------------------------------------------------------------------------
static void overflow_add( World* w, int cid )
{
	w->overflowContacts = grow( w->overflowContacts, &w->overflowCap, w->overflowCount + 1, sizeof( int ) );
	w->contacts[cid].overflowIndex = w->overflowCount;
	w->overflowContacts[w->overflowCount++] = cid;
}

static void overflow_remove( World* w, int cid )
{
	int idx = w->contacts[cid].overflowIndex;
	int last = w->overflowCount - 1;
	if ( idx != last )
	{
		int moved = w->overflowContacts[last];
		w->overflowContacts[idx] = moved;
		w->contacts[moved].overflowIndex = idx;
	}
	w->overflowCount -= 1;
	w->contacts[cid].overflowIndex = P_NULL;
}

void p_add_contact_to_graph( World* w, int cid )
{
	Contact* c = w->contacts + cid;
	Body* a = w->bodies + c->bodyA;
	Body* b = w->bodies + c->bodyB;
	int staticA = a->type == BODY_STATIC;
	int staticB = b->type == BODY_STATIC;
	int color = P_OVERFLOW;
	if ( staticA == 0 && staticB == 0 )
	{
		for ( int i = 0; i < P_OVERFLOW; ++i )
		{
			uint16_t bit = (uint16_t)( 1u << i );
			if ( ( a->colorMask & bit ) || ( b->colorMask & bit ) )
				continue;
			a->colorMask |= bit;
			b->colorMask |= bit;
			color = i;
			break;
		}
	}
	else if ( staticA == 0 )
	{
		for ( int i = 1; i < P_OVERFLOW; ++i )
		{
			uint16_t bit = (uint16_t)( 1u << i );
			if ( a->colorMask & bit )
				continue;
			a->colorMask |= bit;
			color = i;
			break;
		}
	}
	else if ( staticB == 0 )
	{
		for ( int i = 1; i < P_OVERFLOW; ++i )
		{
			uint16_t bit = (uint16_t)( 1u << i );
			if ( b->colorMask & bit )
				continue;
			b->colorMask |= bit;
			color = i;
			break;
		}
	}
	c->color = color;
	if ( color == P_OVERFLOW )
		overflow_add( w, cid );
	// constraint_graph.c:139-181: static bodies contribute zero mass
	if ( staticA )
	{
		c->invMassA = 0.0f;
		c->invIA = 0.0f;
	}
	else
	{
		c->invMassA = a->invMass;
		c->invIA = a->invInertia;
	}
	if ( staticB )
	{
		c->invMassB = 0.0f;
		c->invIB = 0.0f;
	}
	else
	{
		c->invMassB = b->invMass;
		c->invIB = b->invInertia;
	}
}

void p_remove_contact_from_graph( World* w, int cid )
{
	Contact* c = w->contacts + cid;
	int color = c->color;
	if ( color != P_OVERFLOW )
	{
		uint16_t bit = (uint16_t)( 1u << color );
		w->bodies[c->bodyA].colorMask &= (uint16_t)~bit;
		w->bodies[c->bodyB].colorMask &= (uint16_t)~bit;
	}
	else
		overflow_remove( w, cid );
	c->color = P_NULL;
}

static void push_pair( int** arr, int* count, int* cap, int a, int b )
{
	*arr = grow( *arr, cap, 2 * ( *count + 1 ), sizeof( int ) );
	( *arr )[2 * *count] = a;
	( *arr )[2 * *count + 1] = b;
	*count += 1;
}

// contact.c:337-453 b2DestroyContact. During a step the end event joins this
// step's events; between steps (`between`) it waits for the next step's.
static void destroy_contact_ex( World* w, int cid, int wakeBodies, int between )
{
	Contact* c = w->contacts + cid;
	pairset_remove( &w->pairs, pair_key( c->shapeA, c->shapeB ) );
	int touching = c->touchingFlag;
	if ( touching && c->enableContactEvents )
	{
		if ( between )
		{
			ia_push( &w->pendingEnd, c->shapeA );
			ia_push( &w->pendingEnd, c->shapeB );
		}
		else
			push_pair( &w->endEvents, &w->endCount, &w->endCap, c->shapeA, c->shapeB );
	}
	p_contact_edges_unlink( w, cid );
	if ( c->islandId != P_NULL )
		p_unlink_contact( w, cid );
	if ( c->color != P_NULL )
		p_remove_contact_from_graph( w, cid );
	else
		p_set_remove_contact( w, cid );
	int bodyA = c->bodyA, bodyB = c->bodyB;
	c->used = 0;
	c->setIndex = P_NULL;
	free_contact_id( w, cid );
	if ( wakeBodies && touching )
	{
		p_wake_body( w, bodyA );
		p_wake_body( w, bodyB );
	}
}

static void destroy_contact( World* w, int cid )
{
	destroy_contact_ex( w, cid, 0, 0 );
}

// world.c:586-686: serial state changes in contact-id order
static void process_state_changes( World* w )
{
	for ( int id = 0; id < w->contactCount; ++id )
	{
		Contact* c = w->contacts + id;
		if ( c->used == 0 )
			continue;
		uint32_t f = c->simFlags;
		if ( f & SIM_DISJOINT )
		{
			destroy_contact( w, id );
		}
		else if ( f & SIM_STARTED )
		{
			if ( c->enableContactEvents )
			{
				// world.c:630-640: the event carries the manifold of this
				// step's collide phase
				w->beginManifolds =
					grow( w->beginManifolds, &w->beginManifoldCap, 9 * ( w->beginCount + 1 ), sizeof( float ) );
				float* m = w->beginManifolds + 9 * w->beginCount;
				m[0] = c->m.normal.x;
				m[1] = c->m.normal.y;
				m[2] = (float)c->m.pointCount;
				for ( int k = 0; k < 2; ++k )
				{
					int on = k < c->m.pointCount;
					m[3 + 3 * k] = on ? c->m.points[k].point.x : 0.0f;
					m[4 + 3 * k] = on ? c->m.points[k].point.y : 0.0f;
					m[5 + 3 * k] = on ? c->m.points[k].separation : 0.0f;
				}
				push_pair( &w->beginEvents, &w->beginCount, &w->beginCap, c->shapeA, c->shapeB );
			}
			// link first: this wakes a sleeping set the contact touches
			c->touchingFlag = 1;
			p_link_contact( w, id );
			c = w->contacts + id;
			c->simFlags &= ~SIM_STARTED;
			p_add_contact_to_graph( w, id );
		}
		else if ( f & SIM_STOPPED )
		{
			c->simFlags &= ~SIM_STOPPED;
			c->touchingFlag = 0;
			if ( c->enableContactEvents )
				push_pair( &w->endEvents, &w->endCount, &w->endCap, c->shapeA, c->shapeB );
			p_unlink_contact( w, id );
			p_remove_contact_from_graph( w, id );
		}
	}
}

// ---------------------------------------------------------------------------
// step (world.c:695-812)
// ---------------------------------------------------------------------------
double g_portPhase[8];

double p_now( void )
{
	struct timespec t;
	clock_gettime( CLOCK_MONOTONIC, &t );
	return (double)t.tv_sec + 1e-9 * (double)t.tv_nsec;
}

// Batched form: bodies created after this call form a new sub-world with
// the given gravity; shapes of different sub-worlds never make contacts.
int orc_begin_subworld( int wi, double gravityX, double gravityY )
{
	World* w = p_world( wi );
	if ( w == NULL )
		return -1;
	w->subGravity = V( (float)gravityX, (float)gravityY );
	w->subCount += 1;
	return w->subCount - 1;
}

int orc_thread_count( void )
{
#ifdef _OPENMP
	return omp_get_max_threads();
#else
	return 1;
#endif
}

void orc_phase_seconds( double* out8 )
{
	for ( int i = 0; i < 8; ++i )
		out8[i] = g_portPhase[i];
}

void orc_reset_phase_seconds( void )
{
	for ( int i = 0; i < 8; ++i )
		g_portPhase[i] = 0.0;
}

static void* tree_rebuild_thread( void* context )
{
	World* w = context;
	rt_rebuild( w->trees + BODY_DYNAMIC, 0 );
	rt_rebuild( w->trees + BODY_KINEMATIC, 0 );
	return NULL;
}

static void start_tree_rebuild( World* w )
{
	int threads = 1;
#ifdef _OPENMP
	threads = omp_get_max_threads();
#endif
	if ( threads > 1 && pthread_create( &w->treeThread, NULL, tree_rebuild_thread, w ) == 0 )
	{
		w->treeThreadActive = 1;
		w->treeThreadsSaved = threads;
#ifdef _OPENMP
		omp_set_num_threads( threads - 1 );
#endif
		return;
	}
	tree_rebuild_thread( w );
}

// solver.c:1824-1830: the rebuild is finished before the broadphase is
// touched again
void p_finish_tree_rebuild( World* w )
{
	if ( w->treeThreadActive == 0 )
		return;
	pthread_join( w->treeThread, NULL );
	w->treeThreadActive = 0;
#ifdef _OPENMP
	omp_set_num_threads( w->treeThreadsSaved );
#endif
}

void orc_world_step( int wi, double timeStep, int subStepCount )
{
	World* w = p_world( wi );
	w->beginCount = 0;
	w->hitCount = 0;
	w->moveEventCount = 0;
	// end events are double-buffered in the reference and reported for the
	// step that produced them; those made between steps (destroyed contacts
	// and sensors) come first
	w->endCount = 0;
	for ( int i = 0; i + 1 < w->pendingEnd.count; i += 2 )
		push_pair( &w->endEvents, &w->endCount, &w->endCap, w->pendingEnd.data[i], w->pendingEnd.data[i + 1] );
	w->pendingEnd.count = 0;
	w->sensorBegin.count = 0;
	w->sensorEnd.count = 0;
	for ( int i = 0; i < w->pendingSensorEnd.count; ++i )
		ia_push( &w->sensorEnd, w->pendingSensorEnd.data[i] );
	w->pendingSensorEnd.count = 0;
	float dt = (float)timeStep;
	if ( dt == 0.0f )
		return;
	double t0 = p_now();
	update_pairs( w );
	// world.c:488-502 b2Collide -> broad_phase.c:488-492: the dynamic and
	// kinematic trees are rebuilt over their enlarged nodes every step, on a
	// thread of their own as the reference's task does, while the step's
	// parallel loops use one thread fewer (their results do not depend on
	// the thread count); nothing reads those trees before the finalize waits
	// for the rebuild (p_finish_tree_rebuild)
	start_tree_rebuild( w );
	double t1 = p_now();
	int nc = w->contactCount;
#pragma omp parallel for schedule( dynamic, 256 )
	for ( int id = 0; id < nc; ++id )
		if ( w->contacts[id].used && w->contacts[id].setIndex == SET_AWAKE )
			update_contact( w, w->contacts + id );
	double t2 = p_now();
	process_state_changes( w );
	double t3 = p_now();
	g_portPhase[0] += t1 - t0;
	g_portPhase[1] += t2 - t1;
	g_portPhase[2] += t3 - t2;
	p_solve( w, dt, subStepCount < 1 ? 1 : subStepCount );
	p_finish_tree_rebuild( w );
	p_overlap_sensors( w );
}

void orc_set_custom_filter( int wi, orc_custom_filter_fn fn, void* context )
{
	World* w = p_world( wi );
	w->customFilter = fn;
	w->customFilterContext = context;
}

void orc_set_pre_solve( int wi, orc_pre_solve_fn fn, void* context )
{
	World* w = p_world( wi );
	w->preSolve = fn;
	w->preSolveContext = context;
}

// b2World_GetSensorEvents: begin and end (sensor shape, visitor shape) pairs
// of the last step; returns the begin count, the end count in *endCount
int orc_get_sensor_events( int wi, int* begin, int* end, int cap, int* endCount )
{
	World* w = p_world( wi );
	int nb = w->sensorBegin.count / 2, ne = w->sensorEnd.count / 2;
	for ( int i = 0; i < 2 * nb && i < 2 * cap; ++i )
		begin[i] = w->sensorBegin.data[i];
	for ( int i = 0; i < 2 * ne && i < 2 * cap; ++i )
		end[i] = w->sensorEnd.data[i];
	*endCount = ne;
	return nb;
}

double orc_world_step_timed( int wi, double dt, int subSteps, int steps )
{
	struct timespec t0, t1;
	clock_gettime( CLOCK_MONOTONIC, &t0 );
	for ( int i = 0; i < steps; ++i )
		orc_world_step( wi, dt, subSteps );
	clock_gettime( CLOCK_MONOTONIC, &t1 );
	return ( t1.tv_sec - t0.tv_sec ) + 1e-9 * ( t1.tv_nsec - t0.tv_nsec );
}

// ---------------------------------------------------------------------------
// dumps (same layouts as ref_harness.c)
// ---------------------------------------------------------------------------
int orc_body_capacity( int wi )
{
	return p_world( wi )->bodyCount;
}

int orc_get_bodies( int wi, float* out, int cap )
{
	World* w = p_world( wi );
	int n = w->bodyCount < cap ? w->bodyCount : cap;
	for ( int i = 0; i < n; ++i )
	{
		float* o = out + F2D_BODY_DUMP_STRIDE * i;
		memset( o, 0, sizeof( float ) * F2D_BODY_DUMP_STRIDE );
		Body* b = w->bodies + i;
		if ( b->used == 0 )
			continue;
		o[0] = b->xf.p.x;
		o[1] = b->xf.p.y;
		o[2] = b->xf.q.c;
		o[3] = b->xf.q.s;
		o[4] = b->v.x;
		o[5] = b->v.y;
		o[6] = b->w;
		o[7] = b->center.x;
		o[8] = b->center.y;
		o[9] = 1.0f;
		o[10] = (float)b->setIndex;
		o[11] = b->sleepTime;
	}
	return n;
}

int orc_contact_capacity( int wi )
{
	return p_world( wi )->contactCount;
}

int orc_get_contacts( int wi, int* ints, float* floats, int cap )
{
	World* w = p_world( wi );
	int n = 0;
	for ( int id = 0; id < w->contactCount && n < cap; ++id )
	{
		Contact* c = w->contacts + id;
		if ( c->used == 0 )
			continue;
		int* oi = ints + F2D_CONTACT_DUMP_INTS * n;
		float* of = floats + F2D_CONTACT_DUMP_FLOATS * n;
		oi[0] = id;
		oi[1] = c->shapeA;
		oi[2] = c->shapeB;
		oi[3] = c->color;
		oi[4] = c->m.pointCount;
		oi[5] = ( c->touchingFlag ? 1 : 0 ) | ( c->enableContactEvents ? 2 : 0 );
		oi[6] = (int)c->simFlags;
		oi[7] = c->m.points[0].id;
		oi[8] = c->m.points[1].id;
		of[0] = c->m.normal.x;
		of[1] = c->m.normal.y;
		of[2] = c->m.rollingImpulse;
		for ( int k = 0; k < 2; ++k )
		{
			ManifoldPoint* mp = c->m.points + k;
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

int orc_shape_capacity( int wi )
{
	return p_world( wi )->shapeCount;
}

int orc_get_shapes( int wi, float* floats, int* ints, int cap )
{
	World* w = p_world( wi );
	int n = w->shapeCount < cap ? w->shapeCount : cap;
	for ( int i = 0; i < n; ++i )
	{
		Shape* s = w->shapes + i;
		float* f = floats + 8 * i;
		int* k = ints + 4 * i;
		f[0] = s->aabb.lo.x;
		f[1] = s->aabb.lo.y;
		f[2] = s->aabb.hi.x;
		f[3] = s->aabb.hi.y;
		f[4] = s->fatAABB.lo.x;
		f[5] = s->fatAABB.lo.y;
		f[6] = s->fatAABB.hi.x;
		f[7] = s->fatAABB.hi.y;
		k[0] = s->proxyKey;
		k[1] = s->bodyId;
		k[2] = s->g.type;
		k[3] = s->enlarged;
	}
	return n;
}

int orc_get_mass( int wi, float* out, int cap )
{
	World* w = p_world( wi );
	int n = w->bodyCount < cap ? w->bodyCount : cap;
	for ( int i = 0; i < n; ++i )
	{
		float* o = out + 8 * i;
		memset( o, 0, 8 * sizeof( float ) );
		Body* b = w->bodies + i;
		if ( b->used == 0 )
			continue;
		o[0] = b->mass;
		o[1] = b->inertia;
		o[2] = b->invMass;
		o[3] = b->invInertia;
		o[4] = b->localCenter.x;
		o[5] = b->localCenter.y;
		o[6] = b->minExtent;
		o[7] = b->maxExtent;
	}
	return n;
}

int orc_get_polygon( int wi, int shape, float* out )
{
	World* w = p_world( wi );
	Shape* s = w->shapes + shape;
	if ( s->g.type != SHAPE_POLYGON )
		return 0;
	const Polygon* p = &s->g.poly;
	out[0] = (float)p->count;
	out[1] = p->radius;
	out[2] = p->centroid.x;
	out[3] = p->centroid.y;
	for ( int i = 0; i < 8; ++i )
	{
		out[4 + 2 * i] = p->vertices[i].x;
		out[5 + 2 * i] = p->vertices[i].y;
		out[20 + 2 * i] = p->normals[i].x;
		out[21 + 2 * i] = p->normals[i].y;
	}
	return p->count;
}

void orc_get_color_counts( int wi, int* out )
{
	World* w = p_world( wi );
	for ( int i = 0; i < P_COLORS; ++i )
		out[i] = 0;
	for ( int id = 0; id < w->contactCount; ++id )
	{
		Contact* c = w->contacts + id;
		if ( c->used && c->color >= 0 )
			out[c->color] += 1;
	}
	for ( int j = 0; j < w->jointCount; ++j )
	{
		Joint* jt = w->joints + j;
		if ( jt->used && jt->color >= 0 )
			out[jt->color] += 1;
	}
}

// body.c:1480-1510 b2Body_SetAwake
void orc_body_set_awake( int wi, int body, int awake )
{
	World* w = p_world( wi );
	if ( w == NULL || body < 0 || body >= w->bodyCount || w->bodies[body].used == 0 )
		return;
	Body* b = w->bodies + body;
	if ( awake && b->setIndex >= SET_FIRST_SLEEPING )
		p_wake_solver_set( w, b->setIndex );
	else if ( awake == 0 && b->setIndex == SET_AWAKE )
	{
		if ( w->islands[b->islandId].constraintRemoveCount > 0 )
			p_split_island( w, b->islandId );
		p_try_sleep_island( w, w->bodies[body].islandId );
	}
}

// world.c:1715-1740 b2World_EnableSleeping: disabling wakes every set
void orc_world_enable_sleeping( int wi, int enabled )
{
	World* w = p_world( wi );
	if ( w == NULL || ( enabled != 0 ) == ( w->enableSleep != 0 ) )
		return;
	w->enableSleep = enabled != 0;
	if ( enabled == 0 )
		for ( int i = SET_FIRST_SLEEPING; i < w->setCap; ++i )
			if ( w->sets[i].setIndex != P_NULL && w->sets[i].bodies.count > 0 )
				p_wake_solver_set( w, i );
}

int orc_awake_body_count( int wi )
{
	World* w = p_world( wi );
	return w->sets[SET_AWAKE].bodies.count;
}

void orc_event_counts( int wi, int* out )
{
	World* w = p_world( wi );
	out[0] = w->beginCount;
	out[1] = w->endCount;
	out[2] = w->hitCount;
	out[3] = w->moveEventCount;
}

int orc_get_begin_events( int wi, int* pairs, int cap )
{
	World* w = p_world( wi );
	int n = w->beginCount < cap ? w->beginCount : cap;
	memcpy( pairs, w->beginEvents, sizeof( int ) * 2 * (size_t)n );
	return n;
}

// the begin events' manifolds, 9 floats per event (as
// f2d_world_get_begin_manifolds)
int orc_get_begin_manifolds( int wi, float* out9, int cap )
{
	World* w = p_world( wi );
	int n = w->beginCount < cap ? w->beginCount : cap;
	if ( n > 0 )
		memcpy( out9, w->beginManifolds, sizeof( float ) * 9 * (size_t)n );
	return n;
}

int orc_get_end_events( int wi, int* pairs, int cap )
{
	World* w = p_world( wi );
	int n = w->endCount < cap ? w->endCount : cap;
	memcpy( pairs, w->endEvents, sizeof( int ) * 2 * (size_t)n );
	return n;
}

int orc_get_hit_events( int wi, int* ints, float* floats, int cap )
{
	World* w = p_world( wi );
	int n = w->hitCount < cap ? w->hitCount : cap;
	memcpy( ints, w->hitShapes, sizeof( int ) * 2 * (size_t)n );
	memcpy( floats, w->hitData, sizeof( float ) * 5 * (size_t)n );
	return n;
}

int orc_get_move_events( int wi, int* ints, float* floats, int cap )
{
	World* w = p_world( wi );
	int n = w->moveEventCount < cap ? w->moveEventCount : cap;
	for ( int i = 0; i < n; ++i )
	{
		ints[2 * i] = w->moveEventBodies[i];
		ints[2 * i + 1] = w->moveEventAsleep ? w->moveEventAsleep[i] : 0;
	}
	memcpy( floats, w->moveEventXf, sizeof( float ) * 4 * (size_t)n );
	return n;
}

// world-internal helpers used by psolver.c
void p_push_move( World* w, int shapeId )
{
	push_move( w, shapeId );
}

// The restated tree of one body type: leaf shape ids in depth-first visiting
// order, and the node pool's counters (as ref_tree_order / ref_tree_stats)
typedef struct TreeOrderCtx
{
	int* out;
	int cap;
	int n;
} TreeOrderCtx;

static int tree_order_visit( int proxyId, int shape, void* context )
{
	(void)proxyId;
	TreeOrderCtx* c = context;
	if ( c->n < c->cap )
		c->out[c->n] = shape;
	c->n += 1;
	return 1;
}

int orc_tree_order( int wi, int type, int* out, int cap )
{
	const RTree* t = p_world( wi )->trees + type;
	TreeOrderCtx c = { out, cap, 0 };
	if ( t->root != P_NULL )
		rt_query( t, t->nodes[t->root].aabb, ~0ull, tree_order_visit, &c );
	return c.n;
}

void orc_tree_stats( int wi, int type, int* out6 )
{
	const RTree* t = p_world( wi )->trees + type;
	out6[0] = t->count;
	out6[1] = t->cap;
	out6[2] = t->proxyCount;
	out6[3] = t->root == P_NULL ? 0 : t->nodes[t->root].height;
	out6[4] = t->root;
	out6[5] = t->freeList;
}

// Every node of the restated tree of one body type: ints (child1, child2,
// parent, height, flags, shape) and box (lower, upper) per node id; returns
// the node capacity
int orc_tree_nodes( int wi, int type, int* ints, float* boxes, int cap )
{
	const RTree* t = p_world( wi )->trees + type;
	int n = t->cap < cap ? t->cap : cap;
	for ( int i = 0; i < n; ++i )
	{
		const RNode* nd = t->nodes + i;
		int* k = ints + 6 * i;
		k[0] = nd->child1;
		k[1] = nd->child2;
		k[2] = nd->parent;
		k[3] = nd->height;
		k[4] = nd->flags;
		k[5] = nd->shape;
		float* b = boxes + 4 * i;
		b[0] = nd->aabb.lo.x;
		b[1] = nd->aabb.lo.y;
		b[2] = nd->aabb.hi.x;
		b[3] = nd->aabb.hi.y;
	}
	return t->cap;
}

// ---------------------------------------------------------------------------
// destroy path (body.c:343-440, shape.c:230-338, :488-540, joint.c:313-351,
// :702-822, sensor.c:353-380, broad_phase.c:70-114)
// ---------------------------------------------------------------------------
static void free_id( int** freeList, int* freeCount, int id )
{
	*freeList = realloc( *freeList, sizeof( int ) * (size_t)( *freeCount + 1 ) );
	( *freeList )[( *freeCount )++] = id;
}

// broad_phase.c:105-114 b2BroadPhase_DestroyProxy: out of the move array
// (b2UnBufferMove, swap-remove) and out of its tree
static void destroy_proxy( World* w, int sid )
{
	Shape* s = w->shapes + sid;
	if ( s->proxyKey == P_NULL )
		return;
	if ( s->moved )
	{
		for ( int i = 0; i < w->moveCount; ++i )
			if ( w->moveArray[i] == sid )
			{
				w->moveArray[i] = w->moveArray[w->moveCount - 1];
				w->moveCount -= 1;
				break;
			}
		s->moved = 0;
		w->movedFlag[sid] = 0;
	}
	int t = s->proxyKey & 3;
	rt_destroy_proxy( w->trees + t, s->proxyKey >> 2 );
	if ( t == BODY_STATIC )
		w->staticOrderDirty = 1;
	s->proxyKey = P_NULL;
}

// sensor.c:353-380 b2DestroySensor: an end event per current visitor, then
// the sensor leaves the sensor array by swap-remove
static void destroy_sensor( World* w, int sid )
{
	Shape* s = w->shapes + sid;
	int idx = s->sensorIndex;
	PSensor* sn = w->sensors + idx;
	for ( int i = 0; i < sn->overlaps2.count; ++i )
	{
		ia_push( &w->pendingSensorEnd, sid );
		ia_push( &w->pendingSensorEnd, sn->overlaps2.data[i] );
	}
	ia_free( &sn->overlaps1 );
	ia_free( &sn->overlaps2 );
	int last = w->sensorCount - 1;
	if ( idx != last )
	{
		w->sensors[idx] = w->sensors[last];
		w->shapes[w->sensors[idx].shapeId].sensorIndex = idx;
	}
	memset( w->sensors + last, 0, sizeof( PSensor ) );
	w->sensorCount = last;
	s->sensorIndex = P_NULL;
}

// shape.c:230-316 b2DestroyShapeInternal
static void destroy_shape_internal( World* w, int sid, int wakeBodies )
{
	Shape* s = w->shapes + sid;
	Body* b = w->bodies + s->bodyId;
	if ( s->prevShape != P_NULL )
		w->shapes[s->prevShape].nextShape = s->nextShape;
	if ( s->nextShape != P_NULL )
		w->shapes[s->nextShape].prevShape = s->prevShape;
	if ( sid == b->headShape )
		b->headShape = s->nextShape;
	b->shapeCount -= 1;
	destroy_proxy( w, sid );
	for ( int key = b->headContactKey; key != P_NULL; )
	{
		Contact* c = w->contacts + ( key >> 1 );
		int cid = key >> 1;
		key = c->edgeNext[key & 1];
		if ( c->shapeA == sid || c->shapeB == sid )
			destroy_contact_ex( w, cid, wakeBodies, 1 );
	}
	if ( s->sensorIndex != P_NULL )
		destroy_sensor( w, sid );
	free_id( &w->shapeFree, &w->shapeFreeCount, sid );
	s->used = 0;
}

// joint.c:702-806 b2DestroyJointInternal
static void destroy_joint_internal( World* w, int jid, int wakeBodies )
{
	Joint* j = w->joints + jid;
	int ids[2] = { j->bodyA, j->bodyB };
	for ( int e = 0; e < 2; ++e )
	{
		Body* b = w->bodies + ids[e];
		int prev = e == 0 ? j->prevA : j->prevB;
		int next = e == 0 ? j->nextA : j->nextB;
		if ( prev != P_NULL )
		{
			Joint* pj = w->joints + ( prev >> 1 );
			if ( prev & 1 )
				pj->nextB = next;
			else
				pj->nextA = next;
		}
		if ( next != P_NULL )
		{
			Joint* nj = w->joints + ( next >> 1 );
			if ( next & 1 )
				nj->prevB = prev;
			else
				nj->prevA = prev;
		}
		if ( b->headJoint == ( ( jid << 1 ) | e ) )
			b->headJoint = next;
		b->jointCount -= 1;
	}
	if ( j->islandId != P_NULL )
		p_unlink_joint( w, jid );
	if ( j->setIndex == SET_AWAKE )
		p_remove_joint_from_graph( w, jid );
	else
		p_set_remove_joint( w, jid );
	j->setIndex = P_NULL;
	j->color = P_NULL;
	j->used = 0;
	free_id( &w->jointFree, &w->jointFreeCount, jid );
	if ( wakeBodies )
	{
		p_wake_body( w, ids[0] );
		p_wake_body( w, ids[1] );
	}
}

// joint.c:313-351 b2DestroyContactsBetweenBodies: the smaller contact list
// is walked (body B's on a tie), no wake
static void destroy_contacts_between( World* w, int bodyA, int bodyB )
{
	Body* a = w->bodies + bodyA;
	Body* b = w->bodies + bodyB;
	int key, other;
	if ( a->contactCount < b->contactCount )
	{
		key = a->headContactKey;
		other = bodyB;
	}
	else
	{
		key = b->headContactKey;
		other = bodyA;
	}
	while ( key != P_NULL )
	{
		int cid = key >> 1, e = key & 1;
		Contact* c = w->contacts + cid;
		key = c->edgeNext[e];
		int otherBody = ( e ^ 1 ) == 0 ? c->bodyA : c->bodyB;
		if ( otherBody == other )
			destroy_contact_ex( w, cid, 0, 1 );
	}
}

void p_joint_created( World* w, int jid )
{
	Joint* j = w->joints + jid;
	if ( j->collideConnected == 0 )
		destroy_contacts_between( w, j->bodyA, j->bodyB );
}

void orc_destroy_joint( int wi, int jid )
{
	World* w = p_world( wi );
	if ( w == NULL || jid < 0 || jid >= w->jointCount || w->joints[jid].used == 0 )
		return;
	destroy_joint_internal( w, jid, 1 );
}

// shape.c:318-338 b2DestroyShape
void orc_destroy_shape( int wi, int sid, int updateBodyMass )
{
	World* w = p_world( wi );
	if ( w == NULL || sid < 0 || sid >= w->shapeCount || w->shapes[sid].used == 0 )
		return;
	int bodyId = w->shapes[sid].bodyId;
	destroy_shape_internal( w, sid, 1 );
	if ( updateBodyMass )
		update_mass( w, w->bodies + bodyId );
}

// shape.c:488-540 b2DestroyChain
void orc_destroy_chain( int wi, int chainId )
{
	World* w = p_world( wi );
	if ( w == NULL || chainId < 0 || chainId >= w->chainCount || w->chains[chainId].used == 0 )
		return;
	PChain* ch = w->chains + chainId;
	for ( int* link = &w->bodies[ch->bodyId].headChain; *link != P_NULL; link = &w->chains[*link].nextChain )
		if ( *link == chainId )
		{
			*link = ch->nextChain;
			break;
		}
	for ( int i = 0; i < ch->count; ++i )
		destroy_shape_internal( w, ch->shapeIds[i], 1 );
	free( ch->shapeIds );
	ch->shapeIds = NULL;
	ch->count = 0;
	ch->used = 0;
	free_id( &w->chainFree, &w->chainFreeCount, chainId );
}

// body.c:343-440 b2DestroyBody: joints, contacts, shapes (with their
// sensors and proxies), chains, island, solver set, id
void orc_destroy_body( int wi, int bodyId )
{
	World* w = p_world( wi );
	if ( w == NULL || bodyId < 0 || bodyId >= w->bodyCount || w->bodies[bodyId].used == 0 )
		return;
	Body* b = w->bodies + bodyId;
	for ( int key = b->headJoint; key != P_NULL; )
	{
		Joint* j = w->joints + ( key >> 1 );
		int jid = key >> 1;
		key = ( key & 1 ) ? j->nextB : j->nextA;
		destroy_joint_internal( w, jid, 1 );
	}
	for ( int key = b->headContactKey; key != P_NULL; )
	{
		int cid = key >> 1;
		Contact* c = w->contacts + cid;
		key = c->edgeNext[key & 1];
		destroy_contact_ex( w, cid, 1, 1 );
	}
	for ( int sid = b->headShape; sid != P_NULL; sid = w->shapes[sid].nextShape )
	{
		Shape* s = w->shapes + sid;
		if ( s->sensorIndex != P_NULL )
			destroy_sensor( w, sid );
		destroy_proxy( w, sid );
		free_id( &w->shapeFree, &w->shapeFreeCount, sid );
		s->used = 0;
	}
	for ( int c = b->headChain; c != P_NULL; c = w->chains[c].nextChain )
	{
		free( w->chains[c].shapeIds );
		w->chains[c].shapeIds = NULL;
		w->chains[c].count = 0;
		w->chains[c].used = 0;
		free_id( &w->chainFree, &w->chainFreeCount, c );
	}
	b->headChain = P_NULL;
	p_remove_body_from_island( w, bodyId );
	p_set_remove_body( w, bodyId );
	b->used = 0;
	b->headShape = P_NULL;
	b->headJoint = P_NULL;
	b->headContactKey = P_NULL;
	free_id( &w->bodyFree, &w->bodyFreeCount, bodyId );
}

// ---------------------------------------------------------------------------
// type changes, disable and enable (body.c:1036-1282, 1557-1700)
// ---------------------------------------------------------------------------
static Body* live_body( World* w, int bid );

// shape.c:585-601 b2CreateShapeProxy with forcePairCreation: boxes for the
// proxy's type, a leaf of that tree, the proxy buffered as moved
static void create_proxy_forced( World* w, int sid, int proxyType )
{
	Shape* s = w->shapes + sid;
	Body* b = w->bodies + s->bodyId;
	box2 aabb = p_shape_aabb( &s->g, b->xf );
	aabb.lo.x -= P_SPECULATIVE;
	aabb.lo.y -= P_SPECULATIVE;
	aabb.hi.x += P_SPECULATIVE;
	aabb.hi.y += P_SPECULATIVE;
	s->aabb = aabb;
	float margin = proxyType == BODY_STATIC ? P_SPECULATIVE : P_AABB_MARGIN;
	s->fatAABB.lo.x = aabb.lo.x - margin;
	s->fatAABB.lo.y = aabb.lo.y - margin;
	s->fatAABB.hi.x = aabb.hi.x + margin;
	s->fatAABB.hi.y = aabb.hi.y + margin;
	int proxyId = rt_create_proxy( w->trees + proxyType, s->fatAABB, s->categoryBits, sid );
	s->proxyKey = ( proxyId << 2 ) | proxyType;
	if ( proxyType == BODY_STATIC )
		w->staticOrderDirty = 1;
	push_move( w, sid );
}

static void recreate_proxies( World* w, Body* b, int proxyType )
{
	for ( int sid = b->headShape; sid != P_NULL; sid = w->shapes[sid].nextShape )
	{
		destroy_proxy( w, sid );
		create_proxy_forced( w, sid, proxyType );
	}
}

// body.c:1036-1282 b2Body_SetType
void orc_body_set_type( int wi, int bodyId, int type )
{
	World* w = p_world( wi );
	Body* b = live_body( w, bodyId );
	if ( b == NULL || type < BODY_STATIC || type > BODY_DYNAMIC || b->type == type )
		return;
	int original = b->type;
	if ( b->setIndex == SET_DISABLED )
	{
		b->type = type;
		update_mass( w, b );
		return;
	}
	// contacts go without waking the bodies they touched
	for ( int key = b->headContactKey; key != P_NULL; )
	{
		int cid = key >> 1;
		key = w->contacts[cid].edgeNext[key & 1];
		destroy_contact_ex( w, cid, 0, 1 );
	}
	p_wake_body( w, bodyId );
	for ( int key = b->headJoint; key != P_NULL; )
	{
		Joint* j = w->joints + ( key >> 1 );
		key = ( key & 1 ) ? j->nextB : j->nextA;
		if ( j->islandId != P_NULL )
			p_unlink_joint( w, (int)( j - w->joints ) );
		p_wake_body( w, j->bodyA );
		p_wake_body( w, j->bodyB );
	}
	b->type = type;
	if ( original == BODY_STATIC )
	{
		p_transfer_body( w, SET_AWAKE, bodyId );
		p_create_island_for_body( w, SET_AWAKE, bodyId );
		for ( int key = b->headJoint; key != P_NULL; )
		{
			int jid = key >> 1;
			Joint* j = w->joints + jid;
			key = ( key & 1 ) ? j->nextB : j->nextA;
			if ( j->setIndex == SET_STATIC )
				p_transfer_joint( w, SET_AWAKE, jid );
			else if ( j->setIndex == SET_AWAKE )
			{
				// back into the graph for its colour
				p_transfer_joint( w, SET_STATIC, jid );
				p_transfer_joint( w, SET_AWAKE, jid );
			}
		}
		recreate_proxies( w, b, type );
	}
	else if ( type == BODY_STATIC )
	{
		p_transfer_body( w, SET_STATIC, bodyId );
		p_remove_body_from_island( w, bodyId );
		b->isFast = 0;
		for ( int key = b->headJoint; key != P_NULL; )
		{
			int jid = key >> 1;
			Joint* j = w->joints + jid;
			int other = ( key & 1 ) ? j->bodyA : j->bodyB;
			key = ( key & 1 ) ? j->nextB : j->nextA;
			if ( j->setIndex == SET_DISABLED )
				continue;
			p_transfer_joint( w, SET_STATIC, jid );
			if ( w->bodies[other].setIndex != SET_STATIC )
				p_transfer_joint( w, SET_AWAKE, jid );
		}
		recreate_proxies( w, b, BODY_STATIC );
	}
	else
		recreate_proxies( w, b, type );
	for ( int key = b->headJoint; key != P_NULL; )
	{
		int jid = key >> 1;
		Joint* j = w->joints + jid;
		int other = ( key & 1 ) ? j->bodyA : j->bodyB;
		key = ( key & 1 ) ? j->nextB : j->nextA;
		Body* o = w->bodies + other;
		if ( o->setIndex == SET_DISABLED )
			continue;
		if ( b->type == BODY_STATIC && o->type == BODY_STATIC )
			continue;
		p_link_joint( w, jid, 0 );
	}
	p_merge_awake_islands( w );
	update_mass( w, b );
}

// body.c:1557-1626 b2Body_Disable
void orc_body_disable( int wi, int bodyId )
{
	World* w = p_world( wi );
	Body* b = live_body( w, bodyId );
	if ( b == NULL || b->setIndex == SET_DISABLED )
		return;
	for ( int key = b->headContactKey; key != P_NULL; )
	{
		int cid = key >> 1;
		key = w->contacts[cid].edgeNext[key & 1];
		destroy_contact_ex( w, cid, 1, 1 );
	}
	p_remove_body_from_island( w, bodyId );
	for ( int sid = b->headShape; sid != P_NULL; sid = w->shapes[sid].nextShape )
		destroy_proxy( w, sid );
	p_transfer_body( w, SET_DISABLED, bodyId );
	b->enabled = 0;
	for ( int key = b->headJoint; key != P_NULL; )
	{
		int jid = key >> 1;
		Joint* j = w->joints + jid;
		key = ( key & 1 ) ? j->nextB : j->nextA;
		if ( j->setIndex == SET_DISABLED )
			continue;
		if ( j->islandId != P_NULL )
			p_unlink_joint( w, jid );
		p_transfer_joint( w, SET_DISABLED, jid );
	}
}

// body.c:1628-1700 b2Body_Enable
void orc_body_enable( int wi, int bodyId )
{
	World* w = p_world( wi );
	Body* b = live_body( w, bodyId );
	if ( b == NULL || b->setIndex != SET_DISABLED )
		return;
	int setId = b->type == BODY_STATIC ? SET_STATIC : SET_AWAKE;
	p_transfer_body( w, setId, bodyId );
	b->enabled = 1;
	for ( int sid = b->headShape; sid != P_NULL; sid = w->shapes[sid].nextShape )
		create_proxy_forced( w, sid, b->type );
	if ( setId != SET_STATIC )
		p_create_island_for_body( w, setId, bodyId );
	for ( int key = b->headJoint; key != P_NULL; )
	{
		int jid = key >> 1;
		Joint* j = w->joints + jid;
		key = ( key & 1 ) ? j->nextB : j->nextA;
		Body* ba = w->bodies + j->bodyA;
		Body* bb = w->bodies + j->bodyB;
		if ( ba->setIndex == SET_DISABLED || bb->setIndex == SET_DISABLED )
			continue;
		int jointSet;
		if ( ba->setIndex == SET_STATIC && bb->setIndex == SET_STATIC )
			jointSet = SET_STATIC;
		else if ( ba->setIndex == SET_STATIC )
			jointSet = bb->setIndex;
		else
			jointSet = ba->setIndex;
		p_transfer_joint( w, jointSet, jid );
		if ( jointSet != SET_STATIC )
			p_link_joint( w, jid, 0 );
	}
	p_merge_awake_islands( w );
}

// ---------------------------------------------------------------------------
// properties (body.c:1357-1580, shape.c:979-1262, :1476-1530 and the
// setters and getters of revolute_joint.c, prismatic_joint.c,
// wheel_joint.c, distance_joint.c, weld_joint.c, motor_joint.c,
// mouse_joint.c), one get and one set per kind selected by an F2D_*_ code
// ---------------------------------------------------------------------------
static Body* live_body( World* w, int bid )
{
	return ( w != NULL && bid >= 0 && bid < w->bodyCount && w->bodies[bid].used ) ? w->bodies + bid : NULL;
}

static Shape* live_shape( World* w, int sid )
{
	return ( w != NULL && sid >= 0 && sid < w->shapeCount && w->shapes[sid].used ) ? w->shapes + sid : NULL;
}

static Joint* live_joint( World* w, int jid )
{
	return ( w != NULL && jid >= 0 && jid < w->jointCount && w->joints[jid].used ) ? w->joints + jid : NULL;
}

static int valid_f( double v )
{
	float f = (float)v;
	return !isnan( f ) && !isinf( f );
}

double orc_body_get_param( int wi, int bid, int code )
{
	Body* b = live_body( p_world( wi ), bid );
	if ( b == NULL )
		return 0.0;
	switch ( code )
	{
		case F2D_BODY_LINEAR_DAMPING: return b->linearDamping;
		case F2D_BODY_ANGULAR_DAMPING: return b->angularDamping;
		case F2D_BODY_GRAVITY_SCALE: return b->gravityScale;
		case F2D_BODY_BULLET: return b->isBullet;
		case F2D_BODY_FIXED_ROTATION: return b->fixedRotation;
		case F2D_BODY_ENABLED: return b->enabled;
		case F2D_BODY_TYPE: return b->type;
		case F2D_BODY_LOCAL_CENTER_X: return b->localCenter.x;
		case F2D_BODY_LOCAL_CENTER_Y: return b->localCenter.y;
		case F2D_BODY_WORLD_CENTER_X: return b->center.x;
		case F2D_BODY_WORLD_CENTER_Y: return b->center.y;
		default: return 0.0;
	}
}

void orc_body_set_param( int wi, int bid, int code, double value )
{
	World* w = p_world( wi );
	Body* b = live_body( w, bid );
	if ( b == NULL )
		return;
	float v = (float)value;
	switch ( code )
	{
		case F2D_BODY_LINEAR_DAMPING:
			if ( valid_f( value ) && value >= 0.0 )
				b->linearDamping = v;
			break;
		case F2D_BODY_ANGULAR_DAMPING:
			if ( valid_f( value ) && value >= 0.0 )
				b->angularDamping = v;
			break;
		case F2D_BODY_GRAVITY_SCALE:
			if ( valid_f( value ) )
				b->gravityScale = v;
			break;
		case F2D_BODY_BULLET:
			b->isBullet = value != 0.0;
			break;
		case F2D_BODY_FIXED_ROTATION:
			// body.c:1536-1558: the awake state's angular velocity is cleared
			if ( b->fixedRotation != ( value != 0.0 ) )
			{
				b->fixedRotation = value != 0.0;
				if ( b->setIndex == SET_AWAKE )
					b->w = 0.0f;
				update_mass( w, b );
			}
			break;
		default:
			break;
	}
}

void orc_body_set_mass_data( int wi, int bid, double mass, double inertia, double cx, double cy )
{
	Body* b = live_body( p_world( wi ), bid );
	if ( b == NULL )
		return;
	b->mass = (float)mass;
	b->inertia = (float)inertia;
	b->localCenter = V( (float)cx, (float)cy );
	v2 c = xfPoint( b->xf, b->localCenter );
	b->center = c;
	b->center0 = c;
	b->invMass = b->mass > 0.0f ? 1.0f / b->mass : 0.0f;
	b->invInertia = b->inertia > 0.0f ? 1.0f / b->inertia : 0.0f;
}

void orc_body_apply_mass_from_shapes( int wi, int bid )
{
	World* w = p_world( wi );
	Body* b = live_body( w, bid );
	if ( b != NULL )
		update_mass( w, b );
}

double orc_shape_get_param( int wi, int sid, int code )
{
	Shape* s = live_shape( p_world( wi ), sid );
	if ( s == NULL )
		return 0.0;
	switch ( code )
	{
		case F2D_SHAPE_DENSITY: return s->density;
		case F2D_SHAPE_FRICTION: return s->friction;
		case F2D_SHAPE_RESTITUTION: return s->restitution;
		case F2D_SHAPE_SENSOR: return s->isSensor;
		case F2D_SHAPE_SENSOR_EVENTS: return s->enableSensorEvents;
		case F2D_SHAPE_CONTACT_EVENTS: return s->enableContactEvents;
		case F2D_SHAPE_HIT_EVENTS: return s->enableHitEvents;
		case F2D_SHAPE_PRESOLVE_EVENTS: return s->enablePreSolveEvents;
		case F2D_SHAPE_CATEGORY: return (double)(int64_t)s->categoryBits;
		case F2D_SHAPE_MASK: return (double)(int64_t)s->maskBits;
		case F2D_SHAPE_GROUP: return s->groupIndex;
		default: return 0.0;
	}
}

void orc_shape_set_param( int wi, int sid, int code, double value, int flag )
{
	World* w = p_world( wi );
	Shape* s = live_shape( w, sid );
	if ( s == NULL )
		return;
	float v = (float)value;
	int on = value != 0.0;
	switch ( code )
	{
		case F2D_SHAPE_DENSITY:
			// shape.c:1057-1075
			if ( !valid_f( value ) || value < 0.0 || v == s->density )
				return;
			s->density = v;
			if ( flag )
				update_mass( w, w->bodies + s->bodyId );
			break;
		case F2D_SHAPE_FRICTION:
			if ( valid_f( value ) && value >= 0.0 )
				s->friction = v;
			break;
		case F2D_SHAPE_RESTITUTION:
			if ( valid_f( value ) && value >= 0.0 )
				s->restitution = v;
			break;
		case F2D_SHAPE_SENSOR_EVENTS: s->enableSensorEvents = on; break;
		case F2D_SHAPE_CONTACT_EVENTS: s->enableContactEvents = on; break;
		case F2D_SHAPE_HIT_EVENTS: s->enableHitEvents = on; break;
		case F2D_SHAPE_PRESOLVE_EVENTS: s->enablePreSolveEvents = on; break;
		default: break;
	}
}

// shape.c:1185-1262 b2Shape_SetFilter / b2ResetProxy
void orc_shape_set_filter( int wi, int sid, long long categoryBits, long long maskBits, int groupIndex )
{
	World* w = p_world( wi );
	Shape* s = live_shape( w, sid );
	if ( s == NULL )
		return;
	uint64_t cat = (uint64_t)categoryBits, mask = (uint64_t)maskBits;
	if ( cat == s->categoryBits && mask == s->maskBits && groupIndex == s->groupIndex )
		return;
	int destroyProxyFlag = cat != s->categoryBits;
	s->categoryBits = cat;
	s->maskBits = mask;
	s->groupIndex = groupIndex;
	Body* b = w->bodies + s->bodyId;
	for ( int key = b->headContactKey; key != P_NULL; )
	{
		int cid = key >> 1;
		Contact* c = w->contacts + cid;
		key = c->edgeNext[key & 1];
		if ( c->shapeA == sid || c->shapeB == sid )
			destroy_contact_ex( w, cid, 1, 1 );
	}
	int proxyType = s->proxyKey != P_NULL ? ( s->proxyKey & 3 ) : b->type;
	box2 aabb = p_shape_aabb( &s->g, b->xf );
	aabb.lo.x -= P_SPECULATIVE;
	aabb.lo.y -= P_SPECULATIVE;
	aabb.hi.x += P_SPECULATIVE;
	aabb.hi.y += P_SPECULATIVE;
	s->aabb = aabb;
	float margin = proxyType == BODY_STATIC ? P_SPECULATIVE : P_AABB_MARGIN;
	s->fatAABB.lo.x = aabb.lo.x - margin;
	s->fatAABB.lo.y = aabb.lo.y - margin;
	s->fatAABB.hi.x = aabb.hi.x + margin;
	s->fatAABB.hi.y = aabb.hi.y + margin;
	if ( s->proxyKey == P_NULL )
		return;
	if ( destroyProxyFlag )
	{
		destroy_proxy( w, sid );
		int proxyId = rt_create_proxy( w->trees + proxyType, s->fatAABB, s->categoryBits, sid );
		s->proxyKey = ( proxyId << 2 ) | proxyType;
	}
	else
		rt_move_proxy( w->trees + proxyType, s->proxyKey >> 2, s->fatAABB );
	if ( proxyType == BODY_STATIC )
		w->staticOrderDirty = 1;
	push_move( w, sid );
}

// shape.c:979-1001, geometry.c:456-502
int orc_shape_test_point( int wi, int sid, double x, double y )
{
	World* w = p_world( wi );
	Shape* s = live_shape( w, sid );
	if ( s == NULL )
		return 0;
	v2 lp = invXfPoint( w->bodies[s->bodyId].xf, V( (float)x, (float)y ) );
	const Geometry* g = &s->g;
	if ( g->type == SHAPE_CIRCLE )
	{
		v2 d = sub( lp, g->c1 );
		return dot( d, d ) <= g->radius * g->radius;
	}
	if ( g->type == SHAPE_CAPSULE )
	{
		float rr = g->radius * g->radius;
		v2 d = sub( g->c2, g->c1 );
		float dd = dot( d, d );
		if ( dd == 0.0f )
		{
			v2 e = sub( lp, g->c1 );
			return dot( e, e ) <= rr;
		}
		float t = fclampp( dot( sub( lp, g->c1 ), d ) / dd, 0.0f, 1.0f );
		v2 e = sub( lp, mulAdd( g->c1, t, d ) );
		return dot( e, e ) <= rr;
	}
	if ( g->type == SHAPE_POLYGON )
	{
		ShapeProxy pa = p_make_proxy( g->poly.vertices, g->poly.count, 0.0f );
		ShapeProxy pb = p_make_proxy( &lp, 1, 0.0f );
		xform identity = { { 0.0f, 0.0f }, { 1.0f, 0.0f } };
		SimplexCache cache = { 0 };
		v2 pA, pB, n;
		return p_shape_distance( &pa, &pb, identity, identity, &cache, &pA, &pB, &n ) <= g->poly.radius;
	}
	return 0;
}

void orc_chain_set_param( int wi, int chainId, int code, double value )
{
	World* w = p_world( wi );
	if ( w == NULL || chainId < 0 || chainId >= w->chainCount || w->chains[chainId].used == 0 )
		return;
	PChain* ch = w->chains + chainId;
	for ( int i = 0; i < ch->count; ++i )
		orc_shape_set_param( wi, ch->shapeIds[i], code, value, 0 );
}

static float* joint_param_field( Joint* j, int code )
{
	int t = j->type;
	switch ( code )
	{
		case F2D_JP_LOCAL_ANCHOR_AX: return &j->localOriginAnchorA.x;
		case F2D_JP_LOCAL_ANCHOR_AY: return &j->localOriginAnchorA.y;
		case F2D_JP_LOCAL_ANCHOR_BX: return &j->localOriginAnchorB.x;
		case F2D_JP_LOCAL_ANCHOR_BY: return &j->localOriginAnchorB.y;
		case F2D_JP_SPRING_HERTZ:
			return ( t == P_JOINT_REVOLUTE || t == P_JOINT_PRISMATIC || t == P_JOINT_WHEEL || t == P_JOINT_DISTANCE ||
					 t == P_JOINT_MOUSE )
					   ? &j->hertz
					   : NULL;
		case F2D_JP_SPRING_DAMPING:
			return ( t == P_JOINT_REVOLUTE || t == P_JOINT_PRISMATIC || t == P_JOINT_WHEEL || t == P_JOINT_DISTANCE ||
					 t == P_JOINT_MOUSE )
					   ? &j->dampingRatio
					   : NULL;
		case F2D_JP_TARGET:
			return t == P_JOINT_REVOLUTE ? &j->targetAngle : t == P_JOINT_PRISMATIC ? &j->targetTranslation : NULL;
		case F2D_JP_LOWER:
			return t == P_JOINT_REVOLUTE ? &j->lowerAngle
				   : ( t == P_JOINT_PRISMATIC || t == P_JOINT_WHEEL ) ? &j->lowerTranslation
																		: NULL;
		case F2D_JP_UPPER:
			return t == P_JOINT_REVOLUTE ? &j->upperAngle
				   : ( t == P_JOINT_PRISMATIC || t == P_JOINT_WHEEL ) ? &j->upperTranslation
																		: NULL;
		case F2D_JP_MOTOR_SPEED:
			return ( t == P_JOINT_REVOLUTE || t == P_JOINT_PRISMATIC || t == P_JOINT_WHEEL || t == P_JOINT_DISTANCE )
					   ? &j->motorSpeed
					   : NULL;
		case F2D_JP_MAX_MOTOR:
			return ( t == P_JOINT_REVOLUTE || t == P_JOINT_WHEEL )		   ? &j->maxMotorTorque
				   : ( t == P_JOINT_PRISMATIC || t == P_JOINT_DISTANCE ) ? &j->maxMotorForce
																		   : NULL;
		case F2D_JP_LENGTH: return t == P_JOINT_DISTANCE ? &j->length : NULL;
		case F2D_JP_MIN_LENGTH: return t == P_JOINT_DISTANCE ? &j->minLength : NULL;
		case F2D_JP_MAX_LENGTH: return t == P_JOINT_DISTANCE ? &j->maxLength : NULL;
		case F2D_JP_LINEAR_HERTZ: return t == P_JOINT_WELD ? &j->linearHertz : NULL;
		case F2D_JP_LINEAR_DAMPING: return t == P_JOINT_WELD ? &j->linearDampingRatio : NULL;
		case F2D_JP_ANGULAR_HERTZ: return t == P_JOINT_WELD ? &j->angularHertz : NULL;
		case F2D_JP_ANGULAR_DAMPING: return t == P_JOINT_WELD ? &j->angularDampingRatio : NULL;
		case F2D_JP_LINEAR_OFFSET_X: return t == P_JOINT_MOTOR ? &j->linearOffset.x : NULL;
		case F2D_JP_LINEAR_OFFSET_Y: return t == P_JOINT_MOTOR ? &j->linearOffset.y : NULL;
		case F2D_JP_ANGULAR_OFFSET: return t == P_JOINT_MOTOR ? &j->angularOffset : NULL;
		case F2D_JP_MAX_FORCE: return ( t == P_JOINT_MOTOR || t == P_JOINT_MOUSE ) ? &j->maxForce : NULL;
		case F2D_JP_MAX_TORQUE: return t == P_JOINT_MOTOR ? &j->maxTorque : NULL;
		case F2D_JP_CORRECTION: return t == P_JOINT_MOTOR ? &j->correctionFactor : NULL;
		case F2D_JP_TARGET_X: return t == P_JOINT_MOUSE ? &j->targetA.x : NULL;
		case F2D_JP_TARGET_Y: return t == P_JOINT_MOUSE ? &j->targetA.y : NULL;
		default: return NULL;
	}
}

static int* joint_param_flag( Joint* j, int code )
{
	int t = j->type;
	if ( t != P_JOINT_REVOLUTE && t != P_JOINT_PRISMATIC && t != P_JOINT_WHEEL && t != P_JOINT_DISTANCE )
		return NULL;
	return code == F2D_JP_SPRING_ENABLED ? &j->enableSpring
		   : code == F2D_JP_LIMIT_ENABLED ? &j->enableLimit
		   : code == F2D_JP_MOTOR_ENABLED ? &j->enableMotor
										  : NULL;
}

double orc_joint_get_param( int wi, int jid, int code )
{
	World* w = p_world( wi );
	Joint* j = live_joint( w, jid );
	if ( j == NULL )
		return 0.0;
	int t = j->type;
	if ( code == F2D_JP_TYPE )
	{
		// b2JointType values (types.h)
		static const int map[] = { -1, 5, 6, 0, 4, 7, 2, 3, 1 };
		return t >= 0 && t <= 8 ? map[t] : -1;
	}
	int* flag = joint_param_flag( j, code );
	if ( flag )
		return *flag;
	Body* a = w->bodies + j->bodyA;
	Body* b = w->bodies + j->bodyB;
	if ( code == F2D_JP_MOTOR_EFFORT )
		return ( t == P_JOINT_REVOLUTE || t == P_JOINT_PRISMATIC || t == P_JOINT_WHEEL || t == P_JOINT_DISTANCE )
				   ? w->inv_h * j->motorImpulse
				   : 0.0;
	if ( code == F2D_JP_CURRENT )
	{
		if ( t == P_JOINT_REVOLUTE )
			return unwindAngle( relativeAngle( b->xf.q, a->xf.q ) - j->referenceAngle );
		v2 pA = xfPoint( a->xf, j->localOriginAnchorA ), pB = xfPoint( b->xf, j->localOriginAnchorB );
		if ( t == P_JOINT_DISTANCE )
			return length( sub( pB, pA ) );
		if ( t == P_JOINT_PRISMATIC )
			return dot( sub( pB, pA ), rotate( a->xf.q, j->localAxisA ) );
		return 0.0;
	}
	if ( code == F2D_JP_SPEED && t == P_JOINT_PRISMATIC )
	{
		v2 axisA = rotate( a->xf.q, j->localAxisA );
		v2 rA = rotate( a->xf.q, sub( j->localOriginAnchorA, a->localCenter ) );
		v2 rB = rotate( b->xf.q, sub( j->localOriginAnchorB, b->localCenter ) );
		v2 d = add( sub( b->center, a->center ), sub( rB, rA ) );
		int awakeA = a->setIndex == SET_AWAKE, awakeB = b->setIndex == SET_AWAKE;
		v2 vA = awakeA ? a->v : V( 0.0f, 0.0f ), vB = awakeB ? b->v : V( 0.0f, 0.0f );
		float wA = awakeA ? a->w : 0.0f, wB = awakeB ? b->w : 0.0f;
		v2 vRel = sub( add( vB, crossSV( wB, rB ) ), add( vA, crossSV( wA, rA ) ) );
		return dot( d, crossSV( wA, axisA ) ) + dot( axisA, vRel );
	}
	float* f = joint_param_field( j, code );
	return f ? *f : 0.0;
}

void orc_joint_set_param( int wi, int jid, int code, double value, double value2 )
{
	World* w = p_world( wi );
	Joint* j = live_joint( w, jid );
	if ( j == NULL )
		return;
	int t = j->type;
	float v = (float)value, v2 = (float)value2;
	int* flag = joint_param_flag( j, code );
	if ( flag )
	{
		int on = value != 0.0;
		if ( *flag == on )
			return;
		*flag = on;
		if ( code == F2D_JP_SPRING_ENABLED && t != P_JOINT_DISTANCE )
			j->springImpulse = 0.0f;
		else if ( code == F2D_JP_LIMIT_ENABLED && t != P_JOINT_DISTANCE )
			j->lowerImpulse = j->upperImpulse = 0.0f;
		else if ( code == F2D_JP_MOTOR_ENABLED )
			j->motorImpulse = 0.0f;
		return;
	}
	if ( code == F2D_JP_LOWER && ( t == P_JOINT_REVOLUTE || t == P_JOINT_PRISMATIC || t == P_JOINT_WHEEL ) )
	{
		float* lo = joint_param_field( j, F2D_JP_LOWER );
		float* hi = joint_param_field( j, F2D_JP_UPPER );
		if ( v != *lo || v2 != *hi )
		{
			*lo = fminp( v, v2 );
			*hi = fmaxp( v, v2 );
			j->lowerImpulse = j->upperImpulse = 0.0f;
		}
		return;
	}
	if ( t == P_JOINT_DISTANCE && ( code == F2D_JP_LENGTH || code == F2D_JP_MIN_LENGTH ) )
	{
		if ( code == F2D_JP_LENGTH )
			j->length = fclampp( v, P_LINEAR_SLOP, P_HUGE );
		else
		{
			float lo = fclampp( v, P_LINEAR_SLOP, P_HUGE ), hi = fclampp( v2, P_LINEAR_SLOP, P_HUGE );
			j->minLength = fminp( lo, hi );
			j->maxLength = fmaxp( lo, hi );
		}
		j->impulse = j->lowerImpulse = j->upperImpulse = 0.0f;
		return;
	}
	if ( t == P_JOINT_MOTOR && code == F2D_JP_LINEAR_OFFSET_X )
	{
		j->linearOffset = V( v, v2 );
		return;
	}
	if ( code == F2D_JP_UPPER || code == F2D_JP_MAX_LENGTH || code == F2D_JP_LINEAR_OFFSET_Y || code == F2D_JP_TARGET_X ||
		 code == F2D_JP_TARGET_Y || ( code >= F2D_JP_LOCAL_ANCHOR_AX && code <= F2D_JP_LOCAL_ANCHOR_BY ) )
		return;
	float* f = joint_param_field( j, code );
	if ( f == NULL )
		return;
	if ( t == P_JOINT_MOTOR && ( code == F2D_JP_MAX_FORCE || code == F2D_JP_MAX_TORQUE ) )
		v = fmaxp( 0.0f, v );
	else if ( t == P_JOINT_MOTOR && code == F2D_JP_CORRECTION )
		v = fclampp( v, 0.0f, 1.0f );
	*f = v;
}
