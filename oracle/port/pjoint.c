// Revolute joints of the restatement. TEST INFRASTRUCTURE (oracle).
//
// Reference (packages/forge2d/third_party/box2d/src/):
//   joint.c:1348-1352           b2PrepareJoint: constraint softness from
//                               min(60 Hz, 0.25 inv_h) and damping ratio 2
//   revolute_joint.c:202-258    b2PrepareRevoluteJoint
//   revolute_joint.c:261-287    b2WarmStartRevoluteJoint
//   revolute_joint.c:289-457    b2SolveRevoluteJoint (spring, motor, lower and
//                               upper limit, point constraint via b2Solve22)
// A body outside the awake set (static) is read as the identity body state
// and nothing is written back to it (body.h:116 b2_identityBodyState).
#include "port.h"

typedef struct JState
{
	v2 v;
	float w;
	v2 dp;
	rot dq;
} JState;

static int awake_index( const World* w, int body )
{
	const Body* b = w->bodies + body;
	return ( b->used && b->enabled && b->type != BODY_STATIC ) ? body : P_NULL;
}

static JState load_state( const World* w, int index )
{
	JState s;
	if ( index == P_NULL )
	{
		s.v = V( 0.0f, 0.0f );
		s.w = 0.0f;
		s.dp = V( 0.0f, 0.0f );
		s.dq.c = 1.0f;
		s.dq.s = 0.0f;
		return s;
	}
	const Body* b = w->bodies + index;
	s.v = b->v;
	s.w = b->w;
	s.dp = b->dp;
	s.dq = b->dq;
	return s;
}

static void store_velocity( World* w, int index, v2 v, float wv )
{
	if ( index == P_NULL )
		return;
	w->bodies[index].v = v;
	w->bodies[index].w = wv;
}

static void prepare_weld( World* w, Joint* j, float h );
static void prepare_distance( World* w, Joint* j, float h );

void p_prepare_joint( World* w, Joint* j, float h, float inv_h, Softness jointSoftness )
{
	(void)inv_h;
	j->constraintSoftness = jointSoftness;
	if ( j->type != P_JOINT_REVOLUTE )
	{
		// weld_joint.c:83-140, distance_joint.c:158-205: masses, awake
		// indices, world anchors and centre offset as for the revolute
		const Body* a = w->bodies + j->bodyA;
		const Body* b = w->bodies + j->bodyB;
		j->invMassA = a->invMass;
		j->invMassB = b->invMass;
		j->invIA = a->invInertia;
		j->invIB = b->invInertia;
		j->indexA = awake_index( w, j->bodyA );
		j->indexB = awake_index( w, j->bodyB );
		j->anchorA = rotate( a->xf.q, sub( j->localOriginAnchorA, a->localCenter ) );
		j->anchorB = rotate( b->xf.q, sub( j->localOriginAnchorB, b->localCenter ) );
		j->deltaCenter = sub( b->center, a->center );
		if ( j->type == P_JOINT_WELD )
		{
			j->deltaAngle = unwindAngle( relativeAngle( b->xf.q, a->xf.q ) - j->referenceAngle );
			prepare_weld( w, j, h );
		}
		else
			prepare_distance( w, j, h );
		return;
	}
	const Body* a = w->bodies + j->bodyA;
	const Body* b = w->bodies + j->bodyB;
	float mA = a->invMass, iA = a->invInertia;
	float mB = b->invMass, iB = b->invInertia;
	j->invMassA = mA;
	j->invMassB = mB;
	j->invIA = iA;
	j->invIB = iB;
	j->indexA = awake_index( w, j->bodyA );
	j->indexB = awake_index( w, j->bodyB );
	j->anchorA = rotate( a->xf.q, sub( j->localOriginAnchorA, a->localCenter ) );
	j->anchorB = rotate( b->xf.q, sub( j->localOriginAnchorB, b->localCenter ) );
	j->deltaCenter = sub( b->center, a->center );
	j->deltaAngle = relativeAngle( b->xf.q, a->xf.q );
	float k = iA + iB;
	j->axialMass = k > 0.0f ? 1.0f / k : 0.0f;
	j->springSoftness = p_make_soft( j->hertz, j->dampingRatio, h );
	if ( w->enableWarmStarting == 0 )
	{
		j->linearImpulse = V( 0.0f, 0.0f );
		j->springImpulse = 0.0f;
		j->motorImpulse = 0.0f;
		j->lowerImpulse = 0.0f;
		j->upperImpulse = 0.0f;
	}
}

// weld_joint.c:122-140
static void prepare_weld( World* w, Joint* j, float h )
{
	float k = j->invIA + j->invIB;
	j->axialMass = k > 0.0f ? 1.0f / k : 0.0f;
	j->linearSoftness = j->linearHertz == 0.0f ? j->constraintSoftness
												: p_make_soft( j->linearHertz, j->linearDampingRatio, h );
	j->angularSoftness = j->angularHertz == 0.0f ? j->constraintSoftness
												  : p_make_soft( j->angularHertz, j->angularDampingRatio, h );
	if ( w->enableWarmStarting == 0 )
	{
		j->linearImpulse = V( 0.0f, 0.0f );
		j->angularImpulse = 0.0f;
	}
}

// distance_joint.c:185-205
static void prepare_distance( World* w, Joint* j, float h )
{
	float mA = j->invMassA, mB = j->invMassB, iA = j->invIA, iB = j->invIB;
	v2 rA = j->anchorA, rB = j->anchorB;
	v2 separation = add( sub( rB, rA ), j->deltaCenter );
	v2 axis = normalize( separation );
	float crA = cross( rA, axis );
	float crB = cross( rB, axis );
	float k = mA + mB + iA * crA * crA + iB * crB * crB;
	j->axialMass = k > 0.0f ? 1.0f / k : 0.0f;
	j->distanceSoftness = p_make_soft( j->hertz, j->dampingRatio, h );
	if ( w->enableWarmStarting == 0 )
	{
		j->impulse = 0.0f;
		j->lowerImpulse = 0.0f;
		j->upperImpulse = 0.0f;
		j->motorImpulse = 0.0f;
	}
}

// weld_joint.c:142-165
static void warm_weld( World* w, Joint* j )
{
	float mA = j->invMassA, mB = j->invMassB, iA = j->invIA, iB = j->invIB;
	JState sA = load_state( w, j->indexA );
	JState sB = load_state( w, j->indexB );
	v2 rA = rotate( sA.dq, j->anchorA );
	v2 rB = rotate( sB.dq, j->anchorB );
	sA.v = mulSub( sA.v, mA, j->linearImpulse );
	sA.w -= iA * ( cross( rA, j->linearImpulse ) + j->angularImpulse );
	sB.v = mulAdd( sB.v, mB, j->linearImpulse );
	sB.w += iB * ( cross( rB, j->linearImpulse ) + j->angularImpulse );
	store_velocity( w, j->indexA, sA.v, sA.w );
	store_velocity( w, j->indexB, sB.v, sB.w );
}

// distance_joint.c:207-238
static void warm_distance( World* w, Joint* j )
{
	float mA = j->invMassA, mB = j->invMassB, iA = j->invIA, iB = j->invIB;
	JState sA = load_state( w, j->indexA );
	JState sB = load_state( w, j->indexB );
	v2 rA = rotate( sA.dq, j->anchorA );
	v2 rB = rotate( sB.dq, j->anchorB );
	v2 ds = add( sub( sB.dp, sA.dp ), sub( rB, rA ) );
	v2 separation = add( j->deltaCenter, ds );
	v2 axis = normalize( separation );
	float axialImpulse = j->impulse + j->lowerImpulse - j->upperImpulse + j->motorImpulse;
	v2 P = mulSV( axialImpulse, axis );
	sA.v = mulSub( sA.v, mA, P );
	sA.w -= iA * cross( rA, P );
	sB.v = mulAdd( sB.v, mB, P );
	sB.w += iB * cross( rB, P );
	store_velocity( w, j->indexA, sA.v, sA.w );
	store_velocity( w, j->indexB, sB.v, sB.w );
}

// weld_joint.c:167-245
static void solve_weld( World* w, Joint* j, int useBias )
{
	float mA = j->invMassA, mB = j->invMassB, iA = j->invIA, iB = j->invIB;
	JState sA = load_state( w, j->indexA );
	JState sB = load_state( w, j->indexB );
	v2 vA = sA.v, vB = sB.v;
	float wA = sA.w, wB = sB.w;
	{
		float bias = 0.0f, massScale = 1.0f, impulseScale = 0.0f;
		if ( useBias || j->angularHertz > 0.0f )
		{
			float C = relativeAngle( sB.dq, sA.dq ) + j->deltaAngle;
			bias = j->angularSoftness.biasRate * C;
			massScale = j->angularSoftness.massScale;
			impulseScale = j->angularSoftness.impulseScale;
		}
		float Cdot = wB - wA;
		float impulse = -massScale * j->axialMass * ( Cdot + bias ) - impulseScale * j->angularImpulse;
		j->angularImpulse += impulse;
		wA -= iA * impulse;
		wB += iB * impulse;
	}
	{
		v2 rA = rotate( sA.dq, j->anchorA );
		v2 rB = rotate( sB.dq, j->anchorB );
		v2 bias = V( 0.0f, 0.0f );
		float massScale = 1.0f, impulseScale = 0.0f;
		if ( useBias || j->linearHertz > 0.0f )
		{
			v2 C = add( add( sub( sB.dp, sA.dp ), sub( rB, rA ) ), j->deltaCenter );
			bias = mulSV( j->linearSoftness.biasRate, C );
			massScale = j->linearSoftness.massScale;
			impulseScale = j->linearSoftness.impulseScale;
		}
		v2 Cdot = sub( add( vB, crossSV( wB, rB ) ), add( vA, crossSV( wA, rA ) ) );
		v2 cx, cy;
		cx.x = mA + mB + rA.y * rA.y * iA + rB.y * rB.y * iB;
		cy.x = -rA.y * rA.x * iA - rB.y * rB.x * iB;
		cx.y = cy.x;
		cy.y = mA + mB + rA.x * rA.x * iA + rB.x * rB.x * iB;
		v2 b = solve22( cx, cy, add( Cdot, bias ) );
		v2 impulse;
		impulse.x = -massScale * b.x - impulseScale * j->linearImpulse.x;
		impulse.y = -massScale * b.y - impulseScale * j->linearImpulse.y;
		j->linearImpulse = add( j->linearImpulse, impulse );
		vA = mulSub( vA, mA, impulse );
		wA -= iA * cross( rA, impulse );
		vB = mulAdd( vB, mB, impulse );
		wB += iB * cross( rB, impulse );
	}
	store_velocity( w, j->indexA, vA, wA );
	store_velocity( w, j->indexB, vB, wB );
}

// distance_joint.c:240-420
static void solve_distance( World* w, Joint* j, float h, float inv_h, int useBias )
{
	float mA = j->invMassA, mB = j->invMassB, iA = j->invIA, iB = j->invIB;
	JState sA = load_state( w, j->indexA );
	JState sB = load_state( w, j->indexB );
	v2 vA = sA.v, vB = sB.v;
	float wA = sA.w, wB = sB.w;
	v2 rA = rotate( sA.dq, j->anchorA );
	v2 rB = rotate( sB.dq, j->anchorB );
	v2 ds = add( sub( sB.dp, sA.dp ), sub( rB, rA ) );
	v2 separation = add( j->deltaCenter, ds );
	float len = length( separation );
	v2 axis = normalize( separation );
	if ( j->enableSpring && ( j->minLength < j->maxLength || j->enableLimit == 0 ) )
	{
		if ( j->hertz > 0.0f )
		{
			v2 vr = add( sub( vB, vA ), sub( crossSV( wB, rB ), crossSV( wA, rA ) ) );
			float Cdot = dot( axis, vr );
			float C = len - j->length;
			float bias = j->distanceSoftness.biasRate * C;
			float m = j->distanceSoftness.massScale * j->axialMass;
			float impulse = -m * ( Cdot + bias ) - j->distanceSoftness.impulseScale * j->impulse;
			j->impulse += impulse;
			v2 P = mulSV( impulse, axis );
			vA = mulSub( vA, mA, P );
			wA -= iA * cross( rA, P );
			vB = mulAdd( vB, mB, P );
			wB += iB * cross( rB, P );
		}
		if ( j->enableLimit )
		{
			{
				v2 vr = add( sub( vB, vA ), sub( crossSV( wB, rB ), crossSV( wA, rA ) ) );
				float Cdot = dot( axis, vr );
				float C = len - j->minLength;
				float bias = 0.0f, massCoeff = 1.0f, impulseCoeff = 0.0f;
				if ( C > 0.0f )
					bias = C * inv_h;
				else if ( useBias )
				{
					bias = j->constraintSoftness.biasRate * C;
					massCoeff = j->constraintSoftness.massScale;
					impulseCoeff = j->constraintSoftness.impulseScale;
				}
				float impulse = -massCoeff * j->axialMass * ( Cdot + bias ) - impulseCoeff * j->lowerImpulse;
				float newImpulse = fmaxp( 0.0f, j->lowerImpulse + impulse );
				impulse = newImpulse - j->lowerImpulse;
				j->lowerImpulse = newImpulse;
				v2 P = mulSV( impulse, axis );
				vA = mulSub( vA, mA, P );
				wA -= iA * cross( rA, P );
				vB = mulAdd( vB, mB, P );
				wB += iB * cross( rB, P );
			}
			{
				v2 vr = add( sub( vA, vB ), sub( crossSV( wA, rA ), crossSV( wB, rB ) ) );
				float Cdot = dot( axis, vr );
				float C = j->maxLength - len;
				float bias = 0.0f, massScale = 1.0f, impulseScale = 0.0f;
				if ( C > 0.0f )
					bias = C * inv_h;
				else if ( useBias )
				{
					bias = j->constraintSoftness.biasRate * C;
					massScale = j->constraintSoftness.massScale;
					impulseScale = j->constraintSoftness.impulseScale;
				}
				float impulse = -massScale * j->axialMass * ( Cdot + bias ) - impulseScale * j->upperImpulse;
				float newImpulse = fmaxp( 0.0f, j->upperImpulse + impulse );
				impulse = newImpulse - j->upperImpulse;
				j->upperImpulse = newImpulse;
				v2 P = mulSV( -impulse, axis );
				vA = mulSub( vA, mA, P );
				wA -= iA * cross( rA, P );
				vB = mulAdd( vB, mB, P );
				wB += iB * cross( rB, P );
			}
		}
		if ( j->enableMotor )
		{
			v2 vr = add( sub( vB, vA ), sub( crossSV( wB, rB ), crossSV( wA, rA ) ) );
			float Cdot = dot( axis, vr );
			float impulse = j->axialMass * ( j->motorSpeed - Cdot );
			float oldImpulse = j->motorImpulse;
			float maxImpulse = h * j->maxMotorForce;
			j->motorImpulse = fclampp( j->motorImpulse + impulse, -maxImpulse, maxImpulse );
			impulse = j->motorImpulse - oldImpulse;
			v2 P = mulSV( impulse, axis );
			vA = mulSub( vA, mA, P );
			wA -= iA * cross( rA, P );
			vB = mulAdd( vB, mB, P );
			wB += iB * cross( rB, P );
		}
	}
	else
	{
		v2 vr = add( sub( vB, vA ), sub( crossSV( wB, rB ), crossSV( wA, rA ) ) );
		float Cdot = dot( axis, vr );
		float C = len - j->length;
		float bias = 0.0f, massScale = 1.0f, impulseScale = 0.0f;
		if ( useBias )
		{
			bias = j->constraintSoftness.biasRate * C;
			massScale = j->constraintSoftness.massScale;
			impulseScale = j->constraintSoftness.impulseScale;
		}
		float impulse = -massScale * j->axialMass * ( Cdot + bias ) - impulseScale * j->impulse;
		j->impulse += impulse;
		v2 P = mulSV( impulse, axis );
		vA = mulSub( vA, mA, P );
		wA -= iA * cross( rA, P );
		vB = mulAdd( vB, mB, P );
		wB += iB * cross( rB, P );
	}
	store_velocity( w, j->indexA, vA, wA );
	store_velocity( w, j->indexB, vB, wB );
}

void p_warm_start_joint( World* w, Joint* j )
{
	if ( j->type == P_JOINT_WELD )
	{
		warm_weld( w, j );
		return;
	}
	if ( j->type == P_JOINT_DISTANCE )
	{
		warm_distance( w, j );
		return;
	}
	float mA = j->invMassA, mB = j->invMassB, iA = j->invIA, iB = j->invIB;
	JState sA = load_state( w, j->indexA );
	JState sB = load_state( w, j->indexB );
	v2 rA = rotate( sA.dq, j->anchorA );
	v2 rB = rotate( sB.dq, j->anchorB );
	float axialImpulse = j->springImpulse + j->motorImpulse + j->lowerImpulse - j->upperImpulse;
	sA.v = mulSub( sA.v, mA, j->linearImpulse );
	sA.w -= iA * ( cross( rA, j->linearImpulse ) + axialImpulse );
	sB.v = mulAdd( sB.v, mB, j->linearImpulse );
	sB.w += iB * ( cross( rB, j->linearImpulse ) + axialImpulse );
	store_velocity( w, j->indexA, sA.v, sA.w );
	store_velocity( w, j->indexB, sB.v, sB.w );
}

void p_solve_joint( World* w, Joint* j, float h, float inv_h, int useBias )
{
	if ( j->type == P_JOINT_WELD )
	{
		solve_weld( w, j, useBias );
		return;
	}
	if ( j->type == P_JOINT_DISTANCE )
	{
		solve_distance( w, j, h, inv_h, useBias );
		return;
	}
	float mA = j->invMassA, mB = j->invMassB, iA = j->invIA, iB = j->invIB;
	JState sA = load_state( w, j->indexA );
	JState sB = load_state( w, j->indexB );
	v2 vA = sA.v, vB = sB.v;
	float wA = sA.w, wB = sB.w;
	int fixedRotation = ( iA + iB == 0.0f );

	if ( j->enableSpring && fixedRotation == 0 )
	{
		float jointAngle = relativeAngle( sB.dq, sA.dq ) + j->deltaAngle;
		float C = unwindAngle( jointAngle - j->targetAngle );
		float bias = j->springSoftness.biasRate * C;
		float massScale = j->springSoftness.massScale;
		float impulseScale = j->springSoftness.impulseScale;
		float Cdot = wB - wA;
		float impulse = -massScale * j->axialMass * ( Cdot + bias ) - impulseScale * j->springImpulse;
		j->springImpulse += impulse;
		wA -= iA * impulse;
		wB += iB * impulse;
	}

	if ( j->enableMotor && fixedRotation == 0 )
	{
		float Cdot = wB - wA - j->motorSpeed;
		float impulse = -j->axialMass * Cdot;
		float oldImpulse = j->motorImpulse;
		float maxImpulse = h * j->maxMotorTorque;
		j->motorImpulse = fclampp( j->motorImpulse + impulse, -maxImpulse, maxImpulse );
		impulse = j->motorImpulse - oldImpulse;
		wA -= iA * impulse;
		wB += iB * impulse;
	}

	if ( j->enableLimit && fixedRotation == 0 )
	{
		float jointAngle = relativeAngle( sB.dq, sA.dq ) + j->deltaAngle - j->referenceAngle;
		jointAngle = unwindAngle( jointAngle );
		// lower limit
		{
			float C = jointAngle - j->lowerAngle;
			float bias = 0.0f, massScale = 1.0f, impulseScale = 0.0f;
			if ( C > 0.0f )
				bias = C * inv_h;
			else if ( useBias )
			{
				bias = j->constraintSoftness.biasRate * C;
				massScale = j->constraintSoftness.massScale;
				impulseScale = j->constraintSoftness.impulseScale;
			}
			float Cdot = wB - wA;
			float oldImpulse = j->lowerImpulse;
			float impulse = -massScale * j->axialMass * ( Cdot + bias ) - impulseScale * oldImpulse;
			j->lowerImpulse = fmaxp( oldImpulse + impulse, 0.0f );
			impulse = j->lowerImpulse - oldImpulse;
			wA -= iA * impulse;
			wB += iB * impulse;
		}
		// upper limit: signs flipped so that C and the impulse stay positive
		{
			float C = j->upperAngle - jointAngle;
			float bias = 0.0f, massScale = 1.0f, impulseScale = 0.0f;
			if ( C > 0.0f )
				bias = C * inv_h;
			else if ( useBias )
			{
				bias = j->constraintSoftness.biasRate * C;
				massScale = j->constraintSoftness.massScale;
				impulseScale = j->constraintSoftness.impulseScale;
			}
			float Cdot = wA - wB;
			float oldImpulse = j->upperImpulse;
			float impulse = -massScale * j->axialMass * ( Cdot + bias ) - impulseScale * oldImpulse;
			j->upperImpulse = fmaxp( oldImpulse + impulse, 0.0f );
			impulse = j->upperImpulse - oldImpulse;
			wA += iA * impulse;
			wB -= iB * impulse;
		}
	}

	// point-to-point constraint
	{
		v2 rA = rotate( sA.dq, j->anchorA );
		v2 rB = rotate( sB.dq, j->anchorB );
		v2 Cdot = sub( add( vB, crossSV( wB, rB ) ), add( vA, crossSV( wA, rA ) ) );
		v2 bias = V( 0.0f, 0.0f );
		float massScale = 1.0f, impulseScale = 0.0f;
		if ( useBias )
		{
			v2 separation = add( add( sub( sB.dp, sA.dp ), sub( rB, rA ) ), j->deltaCenter );
			bias = mulSV( j->constraintSoftness.biasRate, separation );
			massScale = j->constraintSoftness.massScale;
			impulseScale = j->constraintSoftness.impulseScale;
		}
		v2 cx, cy;
		cx.x = mA + mB + rA.y * rA.y * iA + rB.y * rB.y * iB;
		cy.x = -rA.y * rA.x * iA - rB.y * rB.x * iB;
		cx.y = cy.x;
		cy.y = mA + mB + rA.x * rA.x * iA + rB.x * rB.x * iB;
		v2 b = solve22( cx, cy, add( Cdot, bias ) );
		v2 impulse;
		impulse.x = -massScale * b.x - impulseScale * j->linearImpulse.x;
		impulse.y = -massScale * b.y - impulseScale * j->linearImpulse.y;
		j->linearImpulse.x += impulse.x;
		j->linearImpulse.y += impulse.y;
		vA = mulSub( vA, mA, impulse );
		wA -= iA * cross( rA, impulse );
		vB = mulAdd( vB, mB, impulse );
		wB += iB * cross( rB, impulse );
	}

	store_velocity( w, j->indexA, vA, wA );
	store_velocity( w, j->indexB, vB, wB );
}
