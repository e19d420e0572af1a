// Soft-step solver, integration and body finalisation of the restatement.
// TEST INFRASTRUCTURE (oracle). Reference (packages/forge2d/third_party/
// box2d/src/): solver.c:65-200 (integrate), :543-726 (finalize),
// :929-1160 (stage order), :1190-2051 (b2Solve); contact_solver.c:24-510
// (overflow constraints, scalar operand order) and :1438-2120 (graph-colour
// constraints, whose SIMD lanes use separate mul/add in a fixed order; each
// lane is restated here as scalar code with the same operand order);
// solver.h:140-180 (b2MakeSoft).
#include "port.h"
#ifdef _OPENMP
#include <omp.h>
#endif

#include <stdlib.h>
#include <string.h>

void p_push_move( World* w, int shapeId );
void p_solve_continuous( World* w, int bodyId ); // pccd.c

// solver.h:140-180
Softness p_make_soft( float hertz, float zeta, float h )
{
	Softness s;
	if ( hertz == 0.0f )
	{
		s.biasRate = 0.0f;
		s.massScale = 0.0f;
		s.impulseScale = 0.0f;
		return s;
	}
	float omega = 2.0f * P_PI * hertz;
	float a1 = 2.0f * zeta + h * omega;
	float a2 = h * omega * a1;
	float a3 = 1.0f / ( 1.0f + a2 );
	s.biasRate = omega / a1;
	s.massScale = a2 * a3;
	s.impulseScale = a3;
	return s;
}

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

typedef struct BodyView
{
	v2 v;
	float w;
	v2 dp;
	rot dq;
} BodyView;

static BodyView load_body( World* w, int index )
{
	BodyView b;
	if ( index == P_NULL )
	{
		b.v = V( 0.0f, 0.0f );
		b.w = 0.0f;
		b.dp = V( 0.0f, 0.0f );
		b.dq.c = 1.0f;
		b.dq.s = 0.0f;
		return b;
	}
	Body* body = w->bodies + index;
	b.v = body->v;
	b.w = body->w;
	b.dp = body->dp;
	b.dq = body->dq;
	return b;
}

static void store_velocity( World* w, int index, const BodyView* b )
{
	if ( index == P_NULL )
		return;
	w->bodies[index].v = b->v;
	w->bodies[index].w = b->w;
}

// SSE2 lane semantics of contact_solver.c:558-604 (min/max select the second
// operand unless the first compares strictly less/greater; symmetric clamp
// negates by sign flip).
static inline float lmax( float a, float b )
{
	return a > b ? a : b;
}
static inline float lmin( float a, float b )
{
	return a < b ? a : b;
}
static inline float lsymclamp( float a, float b )
{
	float nb = -b;
	return lmax( nb, lmin( a, b ) );
}

// contact_solver.c:1438-1669 (one lane of b2PrepareContactsTask) and
// :24-156 (b2PrepareOverflowContacts); both compute the same values with
// the same scalar expressions.
static void prepare_contact( World* w, Constraint* k, Contact* c, Softness contactSoftness, Softness staticSoftness,
							 float warmStartScale )
{
	const Manifold* m = &c->m;
	Body* ba = w->bodies + c->bodyA;
	Body* bb = w->bodies + c->bodyB;
	int indexA = ba->type == BODY_STATIC ? P_NULL : c->bodyA;
	int indexB = bb->type == BODY_STATIC ? P_NULL : c->bodyB;
	k->contactId = (int)( c - w->contacts );
	k->indexA = indexA;
	k->indexB = indexB;
	v2 vA = V( 0.0f, 0.0f );
	float wA = 0.0f;
	float mA = c->invMassA;
	float iA = c->invIA;
	if ( indexA != P_NULL )
	{
		vA = ba->v;
		wA = ba->w;
	}
	v2 vB = V( 0.0f, 0.0f );
	float wB = 0.0f;
	float mB = c->invMassB;
	float iB = c->invIB;
	if ( indexB != P_NULL )
	{
		vB = bb->v;
		wB = bb->w;
	}
	k->invMassA = mA;
	k->invMassB = mB;
	k->invIA = iA;
	k->invIB = iB;
	{
		float kk = iA + iB;
		k->rollingMass = kk > 0.0f ? 1.0f / kk : 0.0f;
	}
	Softness soft = ( indexA == P_NULL || indexB == P_NULL ) ? staticSoftness : contactSoftness;
	v2 normal = m->normal;
	k->normal = normal;
	k->friction = c->friction;
	k->tangentSpeed = c->tangentSpeed;
	k->restitution = c->restitution;
	k->rollingResistance = c->rollingResistance;
	k->rollingImpulse = warmStartScale * m->rollingImpulse;
	k->biasRate = soft.biasRate;
	k->massScale = soft.massScale;
	k->impulseScale = soft.impulseScale;
	k->pointCount = m->pointCount;
	v2 tangent = rightPerp( normal );
	for ( int j = 0; j < 2; ++j )
	{
		ConstraintPoint* cp = k->points + j;
		if ( j >= m->pointCount )
		{
			memset( cp, 0, sizeof( *cp ) );
			continue;
		}
		const ManifoldPoint* mp = m->points + j;
		v2 rA = mp->anchorA;
		v2 rB = mp->anchorB;
		cp->anchorA = rA;
		cp->anchorB = rB;
		cp->baseSeparation = mp->separation - dot( sub( rB, rA ), normal );
		cp->normalImpulse = warmStartScale * mp->normalImpulse;
		cp->tangentImpulse = warmStartScale * mp->tangentImpulse;
		cp->totalNormalImpulse = 0.0f;
		float rnA = cross( rA, normal );
		float rnB = cross( rB, normal );
		float kNormal = mA + mB + iA * rnA * rnA + iB * rnB * rnB;
		cp->normalMass = kNormal > 0.0f ? 1.0f / kNormal : 0.0f;
		float rtA = cross( rA, tangent );
		float rtB = cross( rB, tangent );
		float kTangent = mA + mB + iA * rtA * rtA + iB * rtB * rtB;
		cp->tangentMass = kTangent > 0.0f ? 1.0f / kTangent : 0.0f;
		v2 vrA = add( vA, crossSV( wA, rA ) );
		v2 vrB = add( vB, crossSV( wB, rB ) );
		cp->relativeVelocity = dot( normal, sub( vrB, vrA ) );
	}
}

// contact_solver.c:1671-1727 (graph lanes)
static void warm_start_lane( World* w, Constraint* c )
{
	BodyView bA = load_body( w, c->indexA );
	BodyView bB = load_body( w, c->indexB );
	float tx = c->normal.y;
	float ty = 0.0f - c->normal.x;
	for ( int j = 0; j < 2; ++j )
	{
		ConstraintPoint* cp = c->points + j;
		v2 rA = cp->anchorA;
		v2 rB = cp->anchorB;
		float Px = cp->normalImpulse * c->normal.x + cp->tangentImpulse * tx;
		float Py = cp->normalImpulse * c->normal.y + cp->tangentImpulse * ty;
		bA.w = bA.w - c->invIA * ( rA.x * Py - rA.y * Px );
		bA.v.x = bA.v.x - c->invMassA * Px;
		bA.v.y = bA.v.y - c->invMassA * Py;
		bB.w = bB.w + c->invIB * ( rB.x * Py - rB.y * Px );
		bB.v.x = bB.v.x + c->invMassB * Px;
		bB.v.y = bB.v.y + c->invMassB * Py;
	}
	bA.w = bA.w - c->invIA * c->rollingImpulse;
	bB.w = bB.w + c->invIB * c->rollingImpulse;
	store_velocity( w, c->indexA, &bA );
	store_velocity( w, c->indexB, &bB );
}

// contact_solver.c:1729-1967 (graph lanes)
static void solve_lane( World* w, Constraint* c, float inv_h, float minBiasVel, int useBias )
{
	BodyView bA = load_body( w, c->indexA );
	BodyView bB = load_body( w, c->indexB );
	float biasRate, massScale, impulseScale;
	if ( useBias )
	{
		biasRate = c->biasRate;
		massScale = c->massScale;
		impulseScale = c->impulseScale;
	}
	else
	{
		biasRate = 0.0f;
		massScale = 1.0f;
		impulseScale = 0.0f;
	}
	float totalNormalImpulse = 0.0f;
	float dpx = bB.dp.x - bA.dp.x;
	float dpy = bB.dp.y - bA.dp.y;
	v2 n = c->normal;
	for ( int j = 0; j < 2; ++j )
	{
		ConstraintPoint* cp = c->points + j;
		v2 rA = cp->anchorA;
		v2 rB = cp->anchorB;
		float rsAx = bA.dq.c * rA.x - bA.dq.s * rA.y;
		float rsAy = bA.dq.s * rA.x + bA.dq.c * rA.y;
		float rsBx = bB.dq.c * rB.x - bB.dq.s * rB.y;
		float rsBy = bB.dq.s * rB.x + bB.dq.c * rB.y;
		float dsx = dpx + ( rsBx - rsAx );
		float dsy = dpy + ( rsBy - rsAy );
		float s = ( n.x * dsx + n.y * dsy ) + cp->baseSeparation;
		int mask = s > 0.0f;
		float specBias = s * inv_h;
		float softBias = lmax( biasRate * s, minBiasVel );
		float bias = mask ? specBias : softBias;
		float pointMassScale = mask ? 1.0f : massScale;
		float pointImpulseScale = mask ? 0.0f : impulseScale;
		float dvx = ( bB.v.x - bB.w * rB.y ) - ( bA.v.x - bA.w * rA.y );
		float dvy = ( bB.v.y + bB.w * rB.x ) - ( bA.v.y + bA.w * rA.x );
		float vn = dvx * n.x + dvy * n.y;
		float negImpulse = cp->normalMass * ( pointMassScale * ( vn + bias ) ) + pointImpulseScale * cp->normalImpulse;
		float newImpulse = lmax( cp->normalImpulse - negImpulse, 0.0f );
		float impulse = newImpulse - cp->normalImpulse;
		cp->normalImpulse = newImpulse;
		cp->totalNormalImpulse = cp->totalNormalImpulse + newImpulse;
		totalNormalImpulse = totalNormalImpulse + newImpulse;
		float Px = impulse * n.x;
		float Py = impulse * n.y;
		bA.v.x = bA.v.x - c->invMassA * Px;
		bA.v.y = bA.v.y - c->invMassA * Py;
		bA.w = bA.w - c->invIA * ( rA.x * Py - rA.y * Px );
		bB.v.x = bB.v.x + c->invMassB * Px;
		bB.v.y = bB.v.y + c->invMassB * Py;
		bB.w = bB.w + c->invIB * ( rB.x * Py - rB.y * Px );
	}
	float tx = n.y;
	float ty = 0.0f - n.x;
	for ( int j = 0; j < 2; ++j )
	{
		ConstraintPoint* cp = c->points + j;
		v2 rA = cp->anchorA;
		v2 rB = cp->anchorB;
		float dvx = ( bB.v.x - bB.w * rB.y ) - ( bA.v.x - bA.w * rA.y );
		float dvy = ( bB.v.y + bB.w * rB.x ) - ( bA.v.y + bA.w * rA.x );
		float vt = dvx * tx + dvy * ty;
		vt = vt - c->tangentSpeed;
		float negImpulse = cp->tangentMass * vt;
		float maxFriction = c->friction * cp->normalImpulse;
		float newImpulse = cp->tangentImpulse - negImpulse;
		newImpulse = lmax( 0.0f - maxFriction, lmin( newImpulse, maxFriction ) );
		float impulse = newImpulse - cp->tangentImpulse;
		cp->tangentImpulse = newImpulse;
		float Px = impulse * tx;
		float Py = impulse * ty;
		bA.v.x = bA.v.x - c->invMassA * Px;
		bA.v.y = bA.v.y - c->invMassA * Py;
		bA.w = bA.w - c->invIA * ( rA.x * Py - rA.y * Px );
		bB.v.x = bB.v.x + c->invMassB * Px;
		bB.v.y = bB.v.y + c->invMassB * Py;
		bB.w = bB.w + c->invIB * ( rB.x * Py - rB.y * Px );
	}
	{
		float deltaLambda = c->rollingMass * ( bA.w - bB.w );
		float lambda = c->rollingImpulse;
		float maxLambda = c->rollingResistance * totalNormalImpulse;
		c->rollingImpulse = lsymclamp( lambda + deltaLambda, maxLambda );
		deltaLambda = c->rollingImpulse - lambda;
		bA.w = bA.w - c->invIA * deltaLambda;
		bB.w = bB.w + c->invIB * deltaLambda;
	}
	store_velocity( w, c->indexA, &bA );
	store_velocity( w, c->indexB, &bB );
}

// contact_solver.c:1969-2076 (graph lanes; lanes whose restitution is zero are
// left unchanged by the lane mask)
static void restitution_lane( World* w, Constraint* c, float threshold )
{
	if ( c->restitution == 0.0f )
		return;
	BodyView bA = load_body( w, c->indexA );
	BodyView bB = load_body( w, c->indexB );
	v2 n = c->normal;
	for ( int j = 0; j < 2; ++j )
	{
		ConstraintPoint* cp = c->points + j;
		int mask1 = ( cp->relativeVelocity + threshold ) > 0.0f;
		int mask2 = cp->totalNormalImpulse == 0.0f;
		float mass = ( mask1 || mask2 ) ? 0.0f : cp->normalMass;
		v2 rA = cp->anchorA;
		v2 rB = cp->anchorB;
		float dvx = ( bB.v.x - bB.w * rB.y ) - ( bA.v.x - bA.w * rA.y );
		float dvy = ( bB.v.y + bB.w * rB.x ) - ( bA.v.y + bA.w * rA.x );
		float vn = dvx * n.x + dvy * n.y;
		float negImpulse = mass * ( vn + c->restitution * cp->relativeVelocity );
		float newImpulse = lmax( cp->normalImpulse - negImpulse, 0.0f );
		float impulse = newImpulse - cp->normalImpulse;
		cp->normalImpulse = newImpulse;
		float Px = impulse * n.x;
		float Py = impulse * n.y;
		bA.v.x = bA.v.x - c->invMassA * Px;
		bA.v.y = bA.v.y - c->invMassA * Py;
		bA.w = bA.w - c->invIA * ( rA.x * Py - rA.y * Px );
		bB.v.x = bB.v.x + c->invMassB * Px;
		bB.v.y = bB.v.y + c->invMassB * Py;
		bB.w = bB.w + c->invIB * ( rB.x * Py - rB.y * Px );
	}
	store_velocity( w, c->indexA, &bA );
	store_velocity( w, c->indexB, &bB );
}

// contact_solver.c:160-225 (b2WarmStartOverflowContacts)
static void warm_start_overflow( World* w, Constraint* c )
{
	BodyView bA = load_body( w, c->indexA );
	BodyView bB = load_body( w, c->indexB );
	v2 vA = bA.v, vB = bB.v;
	float wA = bA.w, wB = bB.w;
	float mA = c->invMassA, iA = c->invIA, mB = c->invMassB, iB = c->invIB;
	v2 normal = c->normal;
	v2 tangent = rightPerp( normal );
	for ( int j = 0; j < c->pointCount; ++j )
	{
		const ConstraintPoint* cp = c->points + j;
		v2 rA = cp->anchorA;
		v2 rB = cp->anchorB;
		v2 P = add( mulSV( cp->normalImpulse, normal ), mulSV( cp->tangentImpulse, tangent ) );
		wA -= iA * cross( rA, P );
		vA = mulAdd( vA, -mA, P );
		wB += iB * cross( rB, P );
		vB = mulAdd( vB, mB, P );
	}
	wA -= iA * c->rollingImpulse;
	wB += iB * c->rollingImpulse;
	bA.v = vA;
	bA.w = wA;
	bB.v = vB;
	bB.w = wB;
	store_velocity( w, c->indexA, &bA );
	store_velocity( w, c->indexB, &bB );
}

// contact_solver.c:227-380 (b2SolveOverflowContacts)
static void solve_overflow( World* w, Constraint* c, float inv_h, float pushout, int useBias )
{
	float mA = c->invMassA, iA = c->invIA, mB = c->invMassB, iB = c->invIB;
	BodyView sA = load_body( w, c->indexA );
	BodyView sB = load_body( w, c->indexB );
	v2 vA = sA.v;
	float wA = sA.w;
	rot dqA = sA.dq;
	v2 vB = sB.v;
	float wB = sB.w;
	rot dqB = sB.dq;
	v2 dp = sub( sB.dp, sA.dp );
	v2 normal = c->normal;
	v2 tangent = rightPerp( normal );
	float friction = c->friction;
	float totalNormalImpulse = 0.0f;
	for ( int j = 0; j < c->pointCount; ++j )
	{
		ConstraintPoint* cp = c->points + j;
		v2 rA = cp->anchorA;
		v2 rB = cp->anchorB;
		v2 ds = add( dp, sub( rotate( dqB, rB ), rotate( dqA, rA ) ) );
		float s = cp->baseSeparation + dot( ds, normal );
		float velocityBias = 0.0f;
		float massScale = 1.0f;
		float impulseScale = 0.0f;
		if ( s > 0.0f )
			velocityBias = s * inv_h;
		else if ( useBias )
		{
			velocityBias = fmaxp( c->biasRate * s, -pushout );
			massScale = c->massScale;
			impulseScale = c->impulseScale;
		}
		v2 vrA = add( vA, crossSV( wA, rA ) );
		v2 vrB = add( vB, crossSV( wB, rB ) );
		float vn = dot( sub( vrB, vrA ), normal );
		float impulse = -cp->normalMass * massScale * ( vn + velocityBias ) - impulseScale * cp->normalImpulse;
		float newImpulse = fmaxp( cp->normalImpulse + impulse, 0.0f );
		impulse = newImpulse - cp->normalImpulse;
		cp->normalImpulse = newImpulse;
		cp->totalNormalImpulse += newImpulse;
		totalNormalImpulse += newImpulse;
		v2 P = mulSV( impulse, normal );
		vA = mulSub( vA, mA, P );
		wA -= iA * cross( rA, P );
		vB = mulAdd( vB, mB, P );
		wB += iB * cross( rB, P );
	}
	for ( int j = 0; j < c->pointCount; ++j )
	{
		ConstraintPoint* cp = c->points + j;
		v2 rA = cp->anchorA;
		v2 rB = cp->anchorB;
		v2 vrB = add( vB, crossSV( wB, rB ) );
		v2 vrA = add( vA, crossSV( wA, rA ) );
		float vt = dot( sub( vrB, vrA ), tangent ) - c->tangentSpeed;
		float impulse = cp->tangentMass * ( -vt );
		float maxFriction = friction * cp->normalImpulse;
		float newImpulse = fclampp( cp->tangentImpulse + impulse, -maxFriction, maxFriction );
		impulse = newImpulse - cp->tangentImpulse;
		cp->tangentImpulse = newImpulse;
		v2 P = mulSV( impulse, tangent );
		vA = mulSub( vA, mA, P );
		wA -= iA * cross( rA, P );
		vB = mulAdd( vB, mB, P );
		wB += iB * cross( rB, P );
	}
	{
		float deltaLambda = -c->rollingMass * ( wB - wA );
		float lambda = c->rollingImpulse;
		float maxLambda = c->rollingResistance * totalNormalImpulse;
		c->rollingImpulse = fclampp( lambda + deltaLambda, -maxLambda, maxLambda );
		deltaLambda = c->rollingImpulse - lambda;
		wA -= iA * deltaLambda;
		wB += iB * deltaLambda;
	}
	sA.v = vA;
	sA.w = wA;
	sB.v = vB;
	sB.w = wB;
	store_velocity( w, c->indexA, &sA );
	store_velocity( w, c->indexB, &sB );
}

// contact_solver.c:382-478 (b2ApplyOverflowRestitution)
static void restitution_overflow( World* w, Constraint* c, float threshold )
{
	float restitution = c->restitution;
	if ( restitution == 0.0f )
		return;
	float mA = c->invMassA, iA = c->invIA, mB = c->invMassB, iB = c->invIB;
	BodyView sA = load_body( w, c->indexA );
	BodyView sB = load_body( w, c->indexB );
	v2 vA = sA.v, vB = sB.v;
	float wA = sA.w, wB = sB.w;
	v2 normal = c->normal;
	for ( int j = 0; j < c->pointCount; ++j )
	{
		ConstraintPoint* cp = c->points + j;
		if ( cp->relativeVelocity > -threshold || cp->totalNormalImpulse == 0.0f )
			continue;
		v2 rA = cp->anchorA;
		v2 rB = cp->anchorB;
		v2 vrB = add( vB, crossSV( wB, rB ) );
		v2 vrA = add( vA, crossSV( wA, rA ) );
		float vn = dot( sub( vrB, vrA ), normal );
		float impulse = -cp->normalMass * ( vn + restitution * cp->relativeVelocity );
		float newImpulse = fmaxp( cp->normalImpulse + impulse, 0.0f );
		impulse = newImpulse - cp->normalImpulse;
		cp->normalImpulse = newImpulse;
		cp->totalNormalImpulse += impulse;
		v2 P = mulSV( impulse, normal );
		vA = mulSub( vA, mA, P );
		wA -= iA * cross( rA, P );
		vB = mulAdd( vB, mB, P );
		wB += iB * cross( rB, P );
	}
	sA.v = vA;
	sA.w = wA;
	sB.v = vB;
	sB.w = wB;
	store_velocity( w, c->indexA, &sA );
	store_velocity( w, c->indexB, &sB );
}

// contact_solver.c:480-509 and :2078-2120 (b2Store*Impulses)
static void store_impulses( World* w, const Constraint* c, int graphLane )
{
	Contact* ct = w->contacts + c->contactId;
	Manifold* m = &ct->m;
	int n = graphLane ? 2 : m->pointCount;
	for ( int j = 0; j < n; ++j )
	{
		m->points[j].normalImpulse = c->points[j].normalImpulse;
		m->points[j].tangentImpulse = c->points[j].tangentImpulse;
		m->points[j].totalNormalImpulse = c->points[j].totalNormalImpulse;
		m->points[j].normalVelocity = c->points[j].relativeVelocity;
	}
	m->rollingImpulse = c->rollingImpulse;
}

static void push_hit( World* w, int a, int b, v2 point, v2 normal, float speed )
{
	w->hitShapes = grow( w->hitShapes, &w->hitCap, 2 * ( w->hitCount + 1 ), sizeof( int ) );
	w->hitData = grow( w->hitData, &w->hitDataCap, 5 * ( w->hitCount + 1 ), sizeof( float ) );
	w->hitShapes[2 * w->hitCount] = a;
	w->hitShapes[2 * w->hitCount + 1] = b;
	float* d = w->hitData + 5 * w->hitCount;
	d[0] = point.x;
	d[1] = point.y;
	d[2] = normal.x;
	d[3] = normal.y;
	d[4] = speed;
	w->hitCount += 1;
}

// solver.c:65-130 (b2IntegrateVelocitiesTask)
static void integrate_velocities( World* w, Body* b, float h, float maxLinearSpeed, float maxAngularSpeed )
{
	float maxLinearSpeedSq = maxLinearSpeed * maxLinearSpeed;
	float maxAngularSpeedSq = maxAngularSpeed * maxAngularSpeed;
	v2 v = b->v;
	float wv = b->w;
	float linearDamping = 1.0f / ( 1.0f + h * b->linearDamping );
	float angularDamping = 1.0f / ( 1.0f + h * b->angularDamping );
	float gravityScale = b->invMass > 0.0f ? b->gravityScale : 0.0f;
	v2 lvd = add( mulSV( h * b->invMass, b->force ), mulSV( h * gravityScale, w->subCount > 0 ? b->gravity : w->gravity ) );
	float avd = h * b->invInertia * b->torque;
	v = mulAdd( lvd, linearDamping, v );
	wv = avd + angularDamping * wv;
	if ( dot( v, v ) > maxLinearSpeedSq )
	{
		float ratio = maxLinearSpeed / length( v );
		v = mulSV( ratio, v );
		b->isSpeedCapped = 1;
	}
	if ( wv * wv > maxAngularSpeedSq && b->allowFastRotation == 0 )
	{
		float ratio = maxAngularSpeed / fabsp( wv );
		wv *= ratio;
		b->isSpeedCapped = 1;
	}
	b->v = v;
	b->w = wv;
}

static int body_awake( const Body* b )
{
	return b->used && b->setIndex == SET_AWAKE;
}

// solver.c:543-726 (b2FinalizeBodiesTask), excluding island bookkeeping
static void finalize_body( World* w, int id, float dt, float inv_dt )
{
	Body* b = w->bodies + id;
	v2 v = b->v;
	float wv = b->w;
	b->center = add( b->center, b->dp );
	b->xf.q = normalizeRot( mulRot( b->dq, b->xf.q ) );
	float maxVelocity = length( v ) + fabsp( wv ) * b->maxExtent;
	float maxDeltaPosition = length( b->dp ) + fabsp( b->dq.s ) * b->maxExtent;
	float positionSleepFactor = 0.5f;
	float sleepVelocity = fmaxp( maxVelocity, positionSleepFactor * inv_dt * maxDeltaPosition );
	b->dp = V( 0.0f, 0.0f );
	b->dq.c = 1.0f;
	b->dq.s = 0.0f;
	b->xf.p = sub( b->center, rotate( b->xf.q, b->localCenter ) );
	// move event (slot reserved before the parallel finalize)
	{
		w->moveEventBodies[b->moveEventIndex] = id;
		float* x = w->moveEventXf + 4 * b->moveEventIndex;
		x[0] = b->xf.p.x;
		x[1] = b->xf.p.y;
		x[2] = b->xf.q.c;
		x[3] = b->xf.q.s;
	}
	b->force = V( 0.0f, 0.0f );
	b->torque = 0.0f;
	b->isSpeedCapped = 0;
	b->isFast = 0;
	if ( w->enableSleep == 0 || b->enableSleep == 0 || sleepVelocity > b->sleepThreshold )
	{
		b->sleepTime = 0.0f;
		if ( b->type == BODY_DYNAMIC && w->enableContinuous && maxVelocity * dt > 0.5f * b->minExtent )
		{
			b->isFast = 1;
			if ( b->isBullet == 0 )
				p_solve_continuous( w, id );
			// bullets: continuous collision against all bodies runs after
			// finalisation in the reference (solver.c:1915-1988); this port
			// treats them as fast non-bullets
			else
				p_solve_continuous( w, id );
		}
		else
		{
			b->center0 = b->center;
			b->rotation0 = b->xf.q;
		}
	}
	else
	{
		b->center0 = b->center;
		b->rotation0 = b->xf.q;
		b->sleepTime += dt;
	}
	xform transform = b->xf;
	int isFast = b->isFast;
	for ( int s = b->headShape; s != P_NULL; s = w->shapes[s].nextShape )
	{
		Shape* sh = w->shapes + s;
		if ( isFast )
		{
			b->enlargeAABB = 1; // enlarged set bit regardless of AABB change
		}
		else
		{
			box2 aabb = p_shape_aabb( &sh->g, transform );
			aabb.lo.x -= P_SPECULATIVE;
			aabb.lo.y -= P_SPECULATIVE;
			aabb.hi.x += P_SPECULATIVE;
			aabb.hi.y += P_SPECULATIVE;
			sh->aabb = aabb;
			if ( boxContains( sh->fatAABB, aabb ) == 0 )
			{
				box2 fat;
				fat.lo.x = aabb.lo.x - P_AABB_MARGIN;
				fat.lo.y = aabb.lo.y - P_AABB_MARGIN;
				fat.hi.x = aabb.hi.x + P_AABB_MARGIN;
				fat.hi.y = aabb.hi.y + P_AABB_MARGIN;
				sh->fatAABB = fat;
				sh->enlarged = 1;
				b->enlargeAABB = 1;
			}
		}
	}
}

// solver.c:1190-2051 restated without worker stages: the stage order of
// b2SolverTask (solver.c:929-1160) is kept exactly:
//   prepare joints, prepare contacts, overflow prepare;
//   per substep: integrate velocities; warm start (overflow joints, overflow
//   contacts, then colours 0..10); solve (same order); integrate positions;
//   relax (same order);
//   restitution (overflow, colours); store impulses.
void p_solve( World* w, float dt, int subStepCount )
{
	w->stepIndex += 1;
	float inv_dt = 1.0f / dt;
	float h = dt / (float)subStepCount;
	float inv_h = (float)subStepCount * inv_dt;
	w->inv_h = inv_h;
	float contactHertz = fminp( w->contactHertz, 0.125f * inv_h );
	Softness contactSoftness = p_make_soft( contactHertz, w->contactDampingRatio, h );
	Softness staticSoftness = p_make_soft( 2.0f * contactHertz, w->contactDampingRatio, h );
	w->contactSpeed = w->maxContactPushSpeed / staticSoftness.massScale;
	float jointHertz = fminp( 60.0f, 0.25f * inv_h );
	Softness jointSoftness = p_make_soft( jointHertz, 2.0f, h );

	// world.c:709: the step's move events start empty
	w->moveEventCount = 0;
	// continuous collision walks the static tree's order (finalize is parallel)
	p_static_order( w );
	// solver.c:1194-1220: merge islands linked this step; nothing to solve
	// without awake bodies
	p_merge_awake_islands( w );
	int awakeCount = w->sets[SET_AWAKE].bodies.count;
	if ( awakeCount == 0 )
		return;

	double tp0 = p_now();
	// constraint order: overflow first (array order), then each colour's
	// contacts in contact-id order
	int nk = 0;
	w->constraintOrder = grow( w->constraintOrder, &w->constraintOrderCap, w->contactCount + 1, sizeof( int ) );
	int* order = w->constraintOrder;
	for ( int k = 0; k < w->overflowCount; ++k )
		order[nk++] = w->overflowContacts[k];
	int overflowCount = nk;
	int colorStart[P_COLORS + 1];
	{
		int cnt[P_OVERFLOW] = { 0 };
		for ( int id = 0; id < w->contactCount; ++id )
		{
			Contact* c = w->contacts + id;
			if ( c->used && c->color >= 0 && c->color < P_OVERFLOW )
				cnt[c->color] += 1;
		}
		int pos[P_OVERFLOW];
		for ( int color = 0; color < P_OVERFLOW; ++color )
		{
			colorStart[color] = nk;
			pos[color] = nk;
			nk += cnt[color];
		}
		colorStart[P_OVERFLOW] = nk;
		for ( int id = 0; id < w->contactCount; ++id )
		{
			Contact* c = w->contacts + id;
			if ( c->used && c->color >= 0 && c->color < P_OVERFLOW )
				order[pos[c->color]++] = id;
		}
	}
	w->constraints = grow( w->constraints, &w->constraintCap, nk + 1, sizeof( Constraint ) );
	Constraint* K = w->constraints;
	float warmStartScale = w->enableWarmStarting ? 1.0f : 0.0f;
#pragma omp parallel for schedule( static )
	for ( int k = 0; k < nk; ++k )
		prepare_contact( w, K + k, w->contacts + order[k], contactSoftness, staticSoftness, warmStartScale );

	// graph-colour joints per colour (joint-id order)
	w->jointOrder = grow( w->jointOrder, &w->jointOrderCap, w->jointCount + 1, sizeof( int ) );
	int* jorder = w->jointOrder;
	int jStart[P_COLORS + 1];
	{
		int nj = 0;
		for ( int color = 0; color < P_OVERFLOW; ++color )
		{
			jStart[color] = nj;
			for ( int j = 0; j < w->jointCount; ++j )
				if ( w->joints[j].used && w->joints[j].color == color )
					jorder[nj++] = j;
		}
		jStart[P_OVERFLOW] = nj;
	}
	// joints in the constraint graph (colours and overflow)
	int jointCount = w->jointCount;
#pragma omp parallel for schedule( static )
	for ( int j = 0; j < jointCount; ++j )
		if ( w->joints[j].used && w->joints[j].color != P_NULL )
			p_prepare_joint( w, w->joints + j, h, inv_h, jointSoftness );

	double tp1 = p_now();
	float maxAngularSpeed = P_MAX_ROTATION * inv_dt;
	float minBiasVel = -w->contactSpeed;
	int bodyCount = w->bodyCount;
	// One team for all substeps. Within a colour no two constraints share a
	// dynamic body, so each colour's constraints run in parallel; the serial
	// overflow constraints run on one thread; implicit barriers separate the
	// stages exactly where the reference's stage order requires.
#pragma omp parallel
	{
		for ( int i = 0; i < subStepCount; ++i )
		{
#pragma omp for schedule( static )
			for ( int b = 0; b < bodyCount; ++b )
				if ( body_awake( w->bodies + b ) )
					integrate_velocities( w, w->bodies + b, h, w->maximumLinearSpeed, maxAngularSpeed );
			// warm start
#pragma omp single
			{
				for ( int k = 0; k < w->overflowJointCount; ++k )
					p_warm_start_joint( w, w->joints + w->overflowJoints[k] );
				for ( int k = 0; k < overflowCount; ++k )
					warm_start_overflow( w, K + k );
			}
			for ( int color = 0; color < P_OVERFLOW; ++color )
			{
#pragma omp for schedule( static ) nowait
				for ( int q = jStart[color]; q < jStart[color + 1]; ++q )
					p_warm_start_joint( w, w->joints + jorder[q] );
#pragma omp for schedule( static )
				for ( int k = colorStart[color]; k < colorStart[color + 1]; ++k )
					warm_start_lane( w, K + k );
			}
			// solve
#pragma omp single
			{
				for ( int k = 0; k < w->overflowJointCount; ++k )
					p_solve_joint( w, w->joints + w->overflowJoints[k], h, inv_h, 1 );
				for ( int k = 0; k < overflowCount; ++k )
					solve_overflow( w, K + k, inv_h, w->maxContactPushSpeed, 1 );
			}
			for ( int color = 0; color < P_OVERFLOW; ++color )
			{
#pragma omp for schedule( static ) nowait
				for ( int q = jStart[color]; q < jStart[color + 1]; ++q )
					p_solve_joint( w, w->joints + jorder[q], h, inv_h, 1 );
#pragma omp for schedule( static )
				for ( int k = colorStart[color]; k < colorStart[color + 1]; ++k )
					solve_lane( w, K + k, inv_h, minBiasVel, 1 );
			}
			// integrate positions (solver.c:182-200)
#pragma omp for schedule( static )
			for ( int b = 0; b < bodyCount; ++b )
			{
				Body* body = w->bodies + b;
				if ( !body_awake( body ) )
					continue;
				body->dq = integrateRot( body->dq, h * body->w );
				body->dp = mulAdd( body->dp, h, body->v );
			}
			// relax
#pragma omp single
			{
				for ( int k = 0; k < w->overflowJointCount; ++k )
					p_solve_joint( w, w->joints + w->overflowJoints[k], h, inv_h, 0 );
				for ( int k = 0; k < overflowCount; ++k )
					solve_overflow( w, K + k, inv_h, w->maxContactPushSpeed, 0 );
			}
			for ( int color = 0; color < P_OVERFLOW; ++color )
			{
#pragma omp for schedule( static ) nowait
				for ( int q = jStart[color]; q < jStart[color + 1]; ++q )
					p_solve_joint( w, w->joints + jorder[q], h, inv_h, 0 );
#pragma omp for schedule( static )
				for ( int k = colorStart[color]; k < colorStart[color + 1]; ++k )
					solve_lane( w, K + k, inv_h, minBiasVel, 0 );
			}
		}
	}
	double tp2 = p_now();
	// restitution
	for ( int k = 0; k < overflowCount; ++k )
		restitution_overflow( w, K + k, w->restitutionThreshold );
	for ( int color = 0; color < P_OVERFLOW; ++color )
	{
#pragma omp parallel for schedule( static )
		for ( int k = colorStart[color]; k < colorStart[color + 1]; ++k )
			restitution_lane( w, K + k, w->restitutionThreshold );
	}
	// store
	for ( int k = 0; k < overflowCount; ++k )
		store_impulses( w, K + k, 0 );
#pragma omp parallel for schedule( static )
	for ( int k = overflowCount; k < nk; ++k )
		store_impulses( w, K + k, 1 );

	double tp3 = p_now();
	// island split of the previous step's candidate (solver.c:1473-1487,
	// finished before the bodies are finalized)
	if ( w->splitIslandId != P_NULL )
		p_split_island( w, w->splitIslandId );
	w->splitIslandId = P_NULL;
	// finalize bodies; move events in awake-set order, one slot per awake body
	const IntArr* awakeBodies = &w->sets[SET_AWAKE].bodies;
	int awakeIslandCount = w->sets[SET_AWAKE].islands.count;
	{
		int ne = awakeBodies->count;
		for ( int i = 0; i < ne; ++i )
			w->bodies[awakeBodies->data[i]].moveEventIndex = i;
		w->moveEventBodies = grow( w->moveEventBodies, &w->moveEventCap, ne + 1, sizeof( int ) );
		w->moveEventXf = grow( w->moveEventXf, &w->moveEventXfCap, 4 * ( ne + 1 ), sizeof( float ) );
		w->moveEventAsleep = grow( w->moveEventAsleep, &w->moveEventAsleepCap, ne + 1, sizeof( int ) );
		memset( w->moveEventAsleep, 0, sizeof( int ) * (size_t)( ne + 1 ) );
		w->moveEventCount = ne;
	}
#pragma omp parallel for schedule( dynamic, 512 )
	for ( int b = 0; b < bodyCount; ++b )
		if ( body_awake( w->bodies + b ) )
			finalize_body( w, b, dt, inv_dt );
	// island keep-awake bits and the split candidate (solver.c:658-675), in
	// awake-set order as one task context sees them
	unsigned char* awakeIslandBits = (unsigned char*)calloc( (size_t)awakeIslandCount + 1, 1 );
	int splitCandidate = P_NULL;
	{
		float splitSleepTime = 0.0f;
		for ( int i = 0; i < awakeBodies->count; ++i )
		{
			Body* b = w->bodies + awakeBodies->data[i];
			Island* isl = w->islands + b->islandId;
			if ( b->sleepTime < P_TIME_TO_SLEEP )
				awakeIslandBits[isl->localIndex] = 1;
			else if ( isl->constraintRemoveCount > 0 )
			{
				if ( b->sleepTime > splitSleepTime )
				{
					splitCandidate = b->islandId;
					splitSleepTime = b->sleepTime;
				}
			}
		}
	}
	double tp4 = p_now();

	// hit events (solver.c:1758-1818): colours in order, overflow last. Within a
	// colour the reference follows its colour array (append / swap-remove); this
	// port walks contact ids, so the event ORDER inside a colour can differ.
	for ( int pass = 0; pass < 2; ++pass )
	{
		int lo = pass == 0 ? overflowCount : 0;
		int hi = pass == 0 ? nk : overflowCount;
		for ( int k = lo; k < hi; ++k )
		{
			Contact* c = w->contacts + K[k].contactId;
			if ( ( c->simFlags & SIM_HIT_EVENT ) == 0 )
				continue;
			float approach = w->hitEventThreshold;
			int hit = 0;
			v2 point = V( 0.0f, 0.0f );
			for ( int p = 0; p < c->m.pointCount; ++p )
			{
				ManifoldPoint* mp = c->m.points + p;
				float s = -mp->normalVelocity;
				if ( s > approach && mp->totalNormalImpulse > 0.0f )
				{
					approach = s;
					point = mp->point;
					hit = 1;
				}
			}
			if ( hit )
				push_hit( w, c->shapeA, c->shapeB, point, c->m.normal, approach );
		}
	}

	p_finish_tree_rebuild( w );
	// solver.c:1842-1905: enlarge the tree proxies of the flagged bodies and
	// build the move array, in awake-set order (the enlarged-body bitset is
	// indexed by awake-set position), each body's shapes in list order; the
	// tree enlargements themselves commute and run in parallel
	{
		const IntArr* awake = &w->sets[SET_AWAKE].bodies;
		int first = w->moveCount;
		for ( int k = 0; k < awake->count; ++k )
		{
			Body* body = w->bodies + awake->data[k];
			if ( body->enlargeAABB == 0 )
				continue;
			body->enlargeAABB = 0;
			for ( int s = body->headShape; s != P_NULL; s = w->shapes[s].nextShape )
			{
				Shape* sh = w->shapes + s;
				if ( sh->enlarged )
				{
					sh->enlarged = 0;
					p_push_move( w, s );
				}
			}
		}
		int n = w->moveCount - first;
		int* proxies[3] = { NULL, NULL, NULL };
		box2* boxes[3] = { NULL, NULL, NULL };
		int counts[3] = { 0, 0, 0 };
		for ( int t = 1; t < 3; ++t )
		{
			proxies[t] = malloc( sizeof( int ) * (size_t)( n + 1 ) );
			boxes[t] = malloc( sizeof( box2 ) * (size_t)( n + 1 ) );
		}
		for ( int i = first; i < w->moveCount; ++i )
		{
			Shape* sh = w->shapes + w->moveArray[i];
			int t = sh->proxyKey & 3;
			if ( t == BODY_STATIC )
				continue;
			proxies[t][counts[t]] = sh->proxyKey >> 2;
			boxes[t][counts[t]] = sh->fatAABB;
			counts[t] += 1;
		}
		for ( int t = 1; t < 3; ++t )
		{
			rt_enlarge_many( w->trees + t, proxies[t], boxes[t], counts[t] );
			free( proxies[t] );
			free( boxes[t] );
		}
	}
	// island sleeping, last (solver.c:1995-2048)
	if ( w->enableSleep )
		p_sleep_islands( w, awakeIslandBits, splitCandidate );
	free( awakeIslandBits );
	double tp5 = p_now();
	g_portPhase[3] += tp1 - tp0;
	g_portPhase[4] += tp2 - tp1;
	g_portPhase[5] += tp3 - tp2;
	g_portPhase[6] += tp4 - tp3;
	g_portPhase[7] += tp5 - tp4;
}
