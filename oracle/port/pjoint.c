// Joints of the restatement. TEST INFRASTRUCTURE (oracle).
//
// Reference (packages/forge2d/third_party/box2d/src/):
//   joint.c:1348-1470           b2PrepareJoint (constraint softness from
//                               min(60 Hz, 0.25 inv_h) and damping ratio 2),
//                               b2WarmStartJoint, b2SolveJoint type dispatch
//   revolute_joint.c:202-457    revolute: spring, motor, limits, point
//   weld_joint.c:83-245         weld: soft or rigid linear and angular
//   distance_joint.c:158-420    distance: rigid rod or spring, limits, motor
//   prismatic_joint.c:279-604   prismatic: spring, motor, limits, 2x2 block
//   wheel_joint.c:183-488       wheel: motor, spring, limits, point to line
//   motor_joint.c:99-262        motor: clamped angular and linear impulses
//   mouse_joint.c:77-214        mouse: body B pulled to a target
// The filter joint prepares and solves nothing.
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
static void prepare_prismatic( World* w, Joint* j, float h );
static void prepare_wheel( World* w, Joint* j, float h );
static void prepare_motor( World* w, Joint* j );
static void prepare_mouse( World* w, Joint* j, float h );

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
		switch ( j->type )
		{
			case P_JOINT_WELD:
				j->deltaAngle = unwindAngle( relativeAngle( b->xf.q, a->xf.q ) - j->referenceAngle );
				prepare_weld( w, j, h );
				break;
			case P_JOINT_DISTANCE:
				prepare_distance( w, j, h );
				break;
			case P_JOINT_PRISMATIC:
				j->deltaAngle = unwindAngle( relativeAngle( b->xf.q, a->xf.q ) - j->referenceAngle );
				prepare_prismatic( w, j, h );
				break;
			case P_JOINT_WHEEL:
				prepare_wheel( w, j, h );
				break;
			case P_JOINT_MOTOR:
				j->deltaCenter = sub( sub( b->center, a->center ), j->linearOffset );
				j->deltaAngle = relativeAngle( b->xf.q, a->xf.q ) - j->angularOffset;
				prepare_motor( w, j );
				break;
			case P_JOINT_MOUSE:
				prepare_mouse( w, j, h );
				break;
			default: // filter joint: nothing to prepare
				break;
		}
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

// prismatic_joint.c:321-346
static void prepare_prismatic( World* w, Joint* j, float h )
{
	const Body* a = w->bodies + j->bodyA;
	float mA = j->invMassA, mB = j->invMassB, iA = j->invIA, iB = j->invIB;
	j->axisA = rotate( a->xf.q, j->localAxisA );
	v2 rA = j->anchorA, rB = j->anchorB;
	v2 d = add( j->deltaCenter, sub( rB, rA ) );
	float a1 = cross( add( d, rA ), j->axisA );
	float a2 = cross( rB, j->axisA );
	float k = mA + mB + iA * a1 * a1 + iB * a2 * a2;
	j->axialMass = k > 0.0f ? 1.0f / k : 0.0f;
	j->springSoftness = p_make_soft( j->hertz, j->dampingRatio, h );
	if ( w->enableWarmStarting == 0 )
	{
		j->prismaticImpulse = V( 0.0f, 0.0f );
		j->springImpulse = 0.0f;
		j->motorImpulse = 0.0f;
		j->lowerImpulse = 0.0f;
		j->upperImpulse = 0.0f;
	}
}

// wheel_joint.c:224-262
static void prepare_wheel( World* w, Joint* j, float h )
{
	const Body* a = w->bodies + j->bodyA;
	float mA = j->invMassA, mB = j->invMassB, iA = j->invIA, iB = j->invIB;
	j->axisA = rotate( a->xf.q, j->localAxisA );
	v2 rA = j->anchorA, rB = j->anchorB;
	v2 d = add( j->deltaCenter, sub( rB, rA ) );
	v2 axisA = j->axisA;
	v2 perpA = leftPerp( axisA );
	float s1 = cross( add( d, rA ), perpA );
	float s2 = cross( rB, perpA );
	float kp = mA + mB + iA * s1 * s1 + iB * s2 * s2;
	j->perpMass = kp > 0.0f ? 1.0f / kp : 0.0f;
	float a1 = cross( add( d, rA ), axisA );
	float a2 = cross( rB, axisA );
	float ka = mA + mB + iA * a1 * a1 + iB * a2 * a2;
	j->axialMass = ka > 0.0f ? 1.0f / ka : 0.0f;
	j->springSoftness = p_make_soft( j->hertz, j->dampingRatio, h );
	float km = iA + iB;
	j->motorMass = km > 0.0f ? 1.0f / km : 0.0f;
	if ( w->enableWarmStarting == 0 )
	{
		j->perpImpulse = 0.0f;
		j->springImpulse = 0.0f;
		j->motorImpulse = 0.0f;
		j->lowerImpulse = 0.0f;
		j->upperImpulse = 0.0f;
	}
}

// motor_joint.c:142-160
static void prepare_motor( World* w, Joint* j )
{
	float mA = j->invMassA, mB = j->invMassB, iA = j->invIA, iB = j->invIB;
	v2 rA = j->anchorA, rB = j->anchorB;
	v2 cx, cy;
	cx.x = mA + mB + rA.y * rA.y * iA + rB.y * rB.y * iB;
	cx.y = -rA.y * rA.x * iA - rB.y * rB.x * iB;
	cy.x = cx.y;
	cy.y = mA + mB + rA.x * rA.x * iA + rB.x * rB.x * iB;
	inverse22( cx, cy, &j->linearMassCx, &j->linearMassCy );
	float ka = iA + iB;
	j->angularMass = ka > 0.0f ? 1.0f / ka : 0.0f;
	if ( w->enableWarmStarting == 0 )
	{
		j->linearImpulse = V( 0.0f, 0.0f );
		j->angularImpulse = 0.0f;
	}
}

// mouse_joint.c:77-128: body B only; the angular softness is fixed at
// 0.5 Hz, damping ratio 0.1
static void prepare_mouse( World* w, Joint* j, float h )
{
	const Body* b = w->bodies + j->bodyB;
	j->linearSoftness = p_make_soft( j->hertz, j->dampingRatio, h );
	j->angularSoftness = p_make_soft( 0.5f, 0.1f, h );
	v2 rB = j->anchorB;
	float mB = b->invMass, iB = b->invInertia;
	v2 cx, cy;
	cx.x = mB + iB * rB.y * rB.y;
	cx.y = -iB * rB.x * rB.y;
	cy.x = cx.y;
	cy.y = mB + iB * rB.x * rB.x;
	inverse22( cx, cy, &j->linearMassCx, &j->linearMassCy );
	j->deltaCenter = sub( b->center, j->targetA );
	if ( w->enableWarmStarting == 0 )
	{
		j->linearImpulse = V( 0.0f, 0.0f );
		j->angularImpulse = 0.0f;
	}
}

// prismatic_joint.c:349-392
static void warm_prismatic( World* w, Joint* j )
{
	float mA = j->invMassA, mB = j->invMassB, iA = j->invIA, iB = j->invIB;
	JState sA = load_state( w, j->indexA );
	JState sB = load_state( w, j->indexB );
	v2 rA = rotate( sA.dq, j->anchorA );
	v2 rB = rotate( sB.dq, j->anchorB );
	v2 d = add( add( sub( sB.dp, sA.dp ), j->deltaCenter ), sub( rB, rA ) );
	v2 axisA = rotate( sA.dq, j->axisA );
	float a1 = cross( add( d, rA ), axisA );
	float a2 = cross( rB, axisA );
	float axialImpulse = j->springImpulse + j->motorImpulse + j->lowerImpulse - j->upperImpulse;
	v2 perpA = leftPerp( axisA );
	float s1 = cross( add( d, rA ), perpA );
	float s2 = cross( rB, perpA );
	float perpImpulse = j->prismaticImpulse.x;
	float angleImpulse = j->prismaticImpulse.y;
	v2 P = add( mulSV( axialImpulse, axisA ), mulSV( perpImpulse, perpA ) );
	float LA = axialImpulse * a1 + perpImpulse * s1 + angleImpulse;
	float LB = axialImpulse * a2 + perpImpulse * s2 + angleImpulse;
	sA.v = mulSub( sA.v, mA, P );
	sA.w -= iA * LA;
	sB.v = mulAdd( sB.v, mB, P );
	sB.w += iB * LB;
	store_velocity( w, j->indexA, sA.v, sA.w );
	store_velocity( w, j->indexB, sB.v, sB.w );
}

// wheel_joint.c:265-304
static void warm_wheel( World* w, Joint* j )
{
	float mA = j->invMassA, mB = j->invMassB, iA = j->invIA, iB = j->invIB;
	JState sA = load_state( w, j->indexA );
	JState sB = load_state( w, j->indexB );
	v2 rA = rotate( sA.dq, j->anchorA );
	v2 rB = rotate( sB.dq, j->anchorB );
	v2 d = add( add( sub( sB.dp, sA.dp ), j->deltaCenter ), sub( rB, rA ) );
	v2 axisA = rotate( sA.dq, j->axisA );
	v2 perpA = leftPerp( axisA );
	float a1 = cross( add( d, rA ), axisA );
	float a2 = cross( rB, axisA );
	float s1 = cross( add( d, rA ), perpA );
	float s2 = cross( rB, perpA );
	float axialImpulse = j->springImpulse + j->lowerImpulse - j->upperImpulse;
	v2 P = add( mulSV( axialImpulse, axisA ), mulSV( j->perpImpulse, perpA ) );
	float LA = axialImpulse * a1 + j->perpImpulse * s1 + j->motorImpulse;
	float LB = axialImpulse * a2 + j->perpImpulse * s2 + j->motorImpulse;
	sA.v = mulSub( sA.v, mA, P );
	sA.w -= iA * LA;
	sB.v = mulAdd( sB.v, mB, P );
	sB.w += iB * LB;
	store_velocity( w, j->indexA, sA.v, sA.w );
	store_velocity( w, j->indexB, sB.v, sB.w );
}

// motor_joint.c:162-184 (the weld joint's warm start with the motor's
// impulses)
static void warm_motor( World* w, Joint* j )
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

// mouse_joint.c:130-151 (body B's state read without the static check)
static void warm_mouse( World* w, Joint* j )
{
	float mB = j->invMassB, iB = j->invIB;
	JState sB = load_state( w, j->indexB );
	v2 rB = rotate( sB.dq, j->anchorB );
	sB.v = mulAdd( sB.v, mB, j->linearImpulse );
	sB.w += iB * ( cross( rB, j->linearImpulse ) + j->angularImpulse );
	store_velocity( w, j->indexB, sB.v, sB.w );
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

// prismatic_joint.c:394-604
static void solve_prismatic( World* w, Joint* j, float h, float inv_h, int useBias )
{
	float mA = j->invMassA, mB = j->invMassB, iA = j->invIA, iB = j->invIB;
	JState sA = load_state( w, j->indexA );
	JState sB = load_state( w, j->indexB );
	v2 vA = sA.v, vB = sB.v;
	float wA = sA.w, wB = sB.w;
	v2 rA = rotate( sA.dq, j->anchorA );
	v2 rB = rotate( sB.dq, j->anchorB );
	v2 d = add( add( sub( sB.dp, sA.dp ), j->deltaCenter ), sub( rB, rA ) );
	v2 axisA = rotate( sA.dq, j->axisA );
	float translation = dot( axisA, d );
	float a1 = cross( add( d, rA ), axisA );
	float a2 = cross( rB, axisA );
	if ( j->enableSpring )
	{
		float C = translation - j->targetTranslation;
		float bias = j->springSoftness.biasRate * C;
		float massScale = j->springSoftness.massScale;
		float impulseScale = j->springSoftness.impulseScale;
		float Cdot = dot( axisA, sub( vB, vA ) ) + a2 * wB - a1 * wA;
		float deltaImpulse = -massScale * j->axialMass * ( Cdot + bias ) - impulseScale * j->springImpulse;
		j->springImpulse += deltaImpulse;
		v2 P = mulSV( deltaImpulse, axisA );
		float LA = deltaImpulse * a1;
		float LB = deltaImpulse * a2;
		vA = mulSub( vA, mA, P );
		wA -= iA * LA;
		vB = mulAdd( vB, mB, P );
		wB += iB * LB;
	}
	if ( j->enableMotor )
	{
		float Cdot = dot( axisA, sub( vB, vA ) ) + a2 * wB - a1 * wA;
		float impulse = j->axialMass * ( j->motorSpeed - Cdot );
		float oldImpulse = j->motorImpulse;
		float maxImpulse = h * j->maxMotorForce;
		j->motorImpulse = fclampp( j->motorImpulse + impulse, -maxImpulse, maxImpulse );
		impulse = j->motorImpulse - oldImpulse;
		v2 P = mulSV( impulse, axisA );
		float LA = impulse * a1;
		float LB = impulse * a2;
		vA = mulSub( vA, mA, P );
		wA -= iA * LA;
		vB = mulAdd( vB, mB, P );
		wB += iB * LB;
	}
	if ( j->enableLimit )
	{
		{
			float C = translation - j->lowerTranslation;
			float bias = 0.0f, massScale = 1.0f, impulseScale = 0.0f;
			if ( C > 0.0f )
				bias = C * inv_h;
			else if ( useBias )
			{
				bias = j->constraintSoftness.biasRate * C;
				massScale = j->constraintSoftness.massScale;
				impulseScale = j->constraintSoftness.impulseScale;
			}
			float oldImpulse = j->lowerImpulse;
			float Cdot = dot( axisA, sub( vB, vA ) ) + a2 * wB - a1 * wA;
			float impulse = -j->axialMass * massScale * ( Cdot + bias ) - impulseScale * oldImpulse;
			j->lowerImpulse = fmaxp( oldImpulse + impulse, 0.0f );
			impulse = j->lowerImpulse - oldImpulse;
			v2 P = mulSV( impulse, axisA );
			float LA = impulse * a1;
			float LB = impulse * a2;
			vA = mulSub( vA, mA, P );
			wA -= iA * LA;
			vB = mulAdd( vB, mB, P );
			wB += iB * LB;
		}
		{
			float C = j->upperTranslation - translation;
			float bias = 0.0f, massScale = 1.0f, impulseScale = 0.0f;
			if ( C > 0.0f )
				bias = C * inv_h;
			else if ( useBias )
			{
				bias = j->constraintSoftness.biasRate * C;
				massScale = j->constraintSoftness.massScale;
				impulseScale = j->constraintSoftness.impulseScale;
			}
			float oldImpulse = j->upperImpulse;
			float Cdot = dot( axisA, sub( vA, vB ) ) + a1 * wA - a2 * wB;
			float impulse = -j->axialMass * massScale * ( Cdot + bias ) - impulseScale * oldImpulse;
			j->upperImpulse = fmaxp( oldImpulse + impulse, 0.0f );
			impulse = j->upperImpulse - oldImpulse;
			v2 P = mulSV( impulse, axisA );
			float LA = impulse * a1;
			float LB = impulse * a2;
			vA = mulAdd( vA, mA, P );
			wA += iA * LA;
			vB = mulSub( vB, mB, P );
			wB -= iB * LB;
		}
	}
	{
		v2 perpA = leftPerp( axisA );
		float s1 = cross( add( d, rA ), perpA );
		float s2 = cross( rB, perpA );
		v2 Cdot;
		Cdot.x = dot( perpA, sub( vB, vA ) ) + s2 * wB - s1 * wA;
		Cdot.y = wB - wA;
		v2 bias = V( 0.0f, 0.0f );
		float massScale = 1.0f, impulseScale = 0.0f;
		if ( useBias )
		{
			v2 C;
			C.x = dot( perpA, d );
			C.y = relativeAngle( sB.dq, sA.dq ) + j->deltaAngle;
			bias = mulSV( j->constraintSoftness.biasRate, C );
			massScale = j->constraintSoftness.massScale;
			impulseScale = j->constraintSoftness.impulseScale;
		}
		float k11 = mA + mB + iA * s1 * s1 + iB * s2 * s2;
		float k12 = iA * s1 + iB * s2;
		float k22 = iA + iB;
		if ( k22 == 0.0f )
			k22 = 1.0f;
		v2 b = solve22( V( k11, k12 ), V( k12, k22 ), add( Cdot, bias ) );
		v2 impulse;
		impulse.x = -massScale * b.x - impulseScale * j->prismaticImpulse.x;
		impulse.y = -massScale * b.y - impulseScale * j->prismaticImpulse.y;
		j->prismaticImpulse.x += impulse.x;
		j->prismaticImpulse.y += impulse.y;
		v2 P = mulSV( impulse.x, perpA );
		float LA = impulse.x * s1 + impulse.y;
		float LB = impulse.x * s2 + impulse.y;
		vA = mulSub( vA, mA, P );
		wA -= iA * LA;
		vB = mulAdd( vB, mB, P );
		wB += iB * LB;
	}
	store_velocity( w, j->indexA, vA, wA );
	store_velocity( w, j->indexB, vB, wB );
}

// wheel_joint.c:306-488
static void solve_wheel( World* w, Joint* j, float h, float inv_h, int useBias )
{
	float mA = j->invMassA, mB = j->invMassB, iA = j->invIA, iB = j->invIB;
	JState sA = load_state( w, j->indexA );
	JState sB = load_state( w, j->indexB );
	v2 vA = sA.v, vB = sB.v;
	float wA = sA.w, wB = sB.w;
	int fixedRotation = ( iA + iB == 0.0f );
	v2 rA = rotate( sA.dq, j->anchorA );
	v2 rB = rotate( sB.dq, j->anchorB );
	v2 d = add( add( sub( sB.dp, sA.dp ), j->deltaCenter ), sub( rB, rA ) );
	v2 axisA = rotate( sA.dq, j->axisA );
	float translation = dot( axisA, d );
	float a1 = cross( add( d, rA ), axisA );
	float a2 = cross( rB, axisA );
	if ( j->enableMotor && fixedRotation == 0 )
	{
		float Cdot = wB - wA - j->motorSpeed;
		float impulse = -j->motorMass * Cdot;
		float oldImpulse = j->motorImpulse;
		float maxImpulse = h * j->maxMotorTorque;
		j->motorImpulse = fclampp( j->motorImpulse + impulse, -maxImpulse, maxImpulse );
		impulse = j->motorImpulse - oldImpulse;
		wA -= iA * impulse;
		wB += iB * impulse;
	}
	if ( j->enableSpring )
	{
		float C = translation;
		float bias = j->springSoftness.biasRate * C;
		float massScale = j->springSoftness.massScale;
		float impulseScale = j->springSoftness.impulseScale;
		float Cdot = dot( axisA, sub( vB, vA ) ) + a2 * wB - a1 * wA;
		float impulse = -massScale * j->axialMass * ( Cdot + bias ) - impulseScale * j->springImpulse;
		j->springImpulse += impulse;
		v2 P = mulSV( impulse, axisA );
		float LA = impulse * a1;
		float LB = impulse * a2;
		vA = mulSub( vA, mA, P );
		wA -= iA * LA;
		vB = mulAdd( vB, mB, P );
		wB += iB * LB;
	}
	if ( j->enableLimit )
	{
		{
			float C = translation - j->lowerTranslation;
			float bias = 0.0f, massScale = 1.0f, impulseScale = 0.0f;
			if ( C > 0.0f )
				bias = C * inv_h;
			else if ( useBias )
			{
				bias = j->constraintSoftness.biasRate * C;
				massScale = j->constraintSoftness.massScale;
				impulseScale = j->constraintSoftness.impulseScale;
			}
			float Cdot = dot( axisA, sub( vB, vA ) ) + a2 * wB - a1 * wA;
			float impulse = -massScale * j->axialMass * ( Cdot + bias ) - impulseScale * j->lowerImpulse;
			float oldImpulse = j->lowerImpulse;
			j->lowerImpulse = fmaxp( oldImpulse + impulse, 0.0f );
			impulse = j->lowerImpulse - oldImpulse;
			v2 P = mulSV( impulse, axisA );
			float LA = impulse * a1;
			float LB = impulse * a2;
			vA = mulSub( vA, mA, P );
			wA -= iA * LA;
			vB = mulAdd( vB, mB, P );
			wB += iB * LB;
		}
		{
			float C = j->upperTranslation - translation;
			float bias = 0.0f, massScale = 1.0f, impulseScale = 0.0f;
			if ( C > 0.0f )
				bias = C * inv_h;
			else if ( useBias )
			{
				bias = j->constraintSoftness.biasRate * C;
				massScale = j->constraintSoftness.massScale;
				impulseScale = j->constraintSoftness.impulseScale;
			}
			float Cdot = dot( axisA, sub( vA, vB ) ) + a1 * wA - a2 * wB;
			float impulse = -massScale * j->axialMass * ( Cdot + bias ) - impulseScale * j->upperImpulse;
			float oldImpulse = j->upperImpulse;
			j->upperImpulse = fmaxp( oldImpulse + impulse, 0.0f );
			impulse = j->upperImpulse - oldImpulse;
			v2 P = mulSV( impulse, axisA );
			float LA = impulse * a1;
			float LB = impulse * a2;
			vA = mulAdd( vA, mA, P );
			wA += iA * LA;
			vB = mulSub( vB, mB, P );
			wB -= iB * LB;
		}
	}
	{
		v2 perpA = leftPerp( axisA );
		float bias = 0.0f, massScale = 1.0f, impulseScale = 0.0f;
		if ( useBias )
		{
			float C = dot( perpA, d );
			bias = j->constraintSoftness.biasRate * C;
			massScale = j->constraintSoftness.massScale;
			impulseScale = j->constraintSoftness.impulseScale;
		}
		float s1 = cross( add( d, rA ), perpA );
		float s2 = cross( rB, perpA );
		float Cdot = dot( perpA, sub( vB, vA ) ) + s2 * wB - s1 * wA;
		float impulse = -massScale * j->perpMass * ( Cdot + bias ) - impulseScale * j->perpImpulse;
		j->perpImpulse += impulse;
		v2 P = mulSV( impulse, perpA );
		float LA = impulse * s1;
		float LB = impulse * s2;
		vA = mulSub( vA, mA, P );
		wA -= iA * LA;
		vB = mulAdd( vB, mB, P );
		wB += iB * LB;
	}
	store_velocity( w, j->indexA, vA, wA );
	store_velocity( w, j->indexB, vB, wB );
}

// motor_joint.c:186-262
static void solve_motor( World* w, Joint* j, float h, float inv_h )
{
	float mA = j->invMassA, mB = j->invMassB, iA = j->invIA, iB = j->invIB;
	JState sA = load_state( w, j->indexA );
	JState sB = load_state( w, j->indexB );
	v2 vA = sA.v, vB = sB.v;
	float wA = sA.w, wB = sB.w;
	{
		float angularSeparation = relativeAngle( sB.dq, sA.dq ) + j->deltaAngle;
		angularSeparation = unwindAngle( angularSeparation );
		float angularBias = inv_h * j->correctionFactor * angularSeparation;
		float Cdot = wB - wA;
		float impulse = -j->angularMass * ( Cdot + angularBias );
		float oldImpulse = j->angularImpulse;
		float maxImpulse = h * j->maxTorque;
		j->angularImpulse = fclampp( j->angularImpulse + impulse, -maxImpulse, maxImpulse );
		impulse = j->angularImpulse - oldImpulse;
		wA -= iA * impulse;
		wB += iB * impulse;
	}
	{
		v2 rA = rotate( sA.dq, j->anchorA );
		v2 rB = rotate( sB.dq, j->anchorB );
		v2 ds = add( sub( sB.dp, sA.dp ), sub( rB, rA ) );
		v2 linearSeparation = add( j->deltaCenter, ds );
		v2 linearBias = mulSV( inv_h * j->correctionFactor, linearSeparation );
		v2 Cdot = sub( add( vB, crossSV( wB, rB ) ), add( vA, crossSV( wA, rA ) ) );
		v2 b = mulMV( j->linearMassCx, j->linearMassCy, add( Cdot, linearBias ) );
		v2 impulse = V( -b.x, -b.y );
		v2 oldImpulse = j->linearImpulse;
		float maxImpulse = h * j->maxForce;
		j->linearImpulse = add( j->linearImpulse, impulse );
		if ( lengthSq( j->linearImpulse ) > maxImpulse * maxImpulse )
		{
			j->linearImpulse = normalize( j->linearImpulse );
			j->linearImpulse.x *= maxImpulse;
			j->linearImpulse.y *= maxImpulse;
		}
		impulse = sub( j->linearImpulse, oldImpulse );
		vA = mulSub( vA, mA, impulse );
		wA -= iA * cross( rA, impulse );
		vB = mulAdd( vB, mB, impulse );
		wB += iB * cross( rB, impulse );
	}
	store_velocity( w, j->indexA, vA, wA );
	store_velocity( w, j->indexB, vB, wB );
}

// mouse_joint.c:153-214
static void solve_mouse( World* w, Joint* j, float h )
{
	float mB = j->invMassB, iB = j->invIB;
	JState sB = load_state( w, j->indexB );
	v2 vB = sB.v;
	float wB = sB.w;
	{
		float massScale = j->angularSoftness.massScale;
		float impulseScale = j->angularSoftness.impulseScale;
		float impulse = iB > 0.0f ? -wB / iB : 0.0f;
		impulse = massScale * impulse - impulseScale * j->angularImpulse;
		j->angularImpulse += impulse;
		wB += iB * impulse;
	}
	float maxImpulse = j->maxForce * h;
	{
		v2 rB = rotate( sB.dq, j->anchorB );
		v2 Cdot = add( vB, crossSV( wB, rB ) );
		v2 separation = add( add( sB.dp, rB ), j->deltaCenter );
		v2 bias = mulSV( j->linearSoftness.biasRate, separation );
		float massScale = j->linearSoftness.massScale;
		float impulseScale = j->linearSoftness.impulseScale;
		v2 b = mulMV( j->linearMassCx, j->linearMassCy, add( Cdot, bias ) );
		v2 impulse;
		impulse.x = -massScale * b.x - impulseScale * j->linearImpulse.x;
		impulse.y = -massScale * b.y - impulseScale * j->linearImpulse.y;
		v2 oldImpulse = j->linearImpulse;
		j->linearImpulse.x += impulse.x;
		j->linearImpulse.y += impulse.y;
		float mag = length( j->linearImpulse );
		if ( mag > maxImpulse )
			j->linearImpulse = mulSV( maxImpulse, normalize( j->linearImpulse ) );
		impulse.x = j->linearImpulse.x - oldImpulse.x;
		impulse.y = j->linearImpulse.y - oldImpulse.y;
		vB = mulAdd( vB, mB, impulse );
		wB += iB * cross( rB, impulse );
	}
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
	switch ( j->type )
	{
		case P_JOINT_WELD:
			warm_weld( w, j );
			return;
		case P_JOINT_DISTANCE:
			warm_distance( w, j );
			return;
		case P_JOINT_PRISMATIC:
			warm_prismatic( w, j );
			return;
		case P_JOINT_WHEEL:
			warm_wheel( w, j );
			return;
		case P_JOINT_MOTOR:
			warm_motor( w, j );
			return;
		case P_JOINT_MOUSE:
			warm_mouse( w, j );
			return;
		case P_JOINT_FILTER:
			return;
		default:
			break;
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
	switch ( j->type )
	{
		case P_JOINT_WELD:
			solve_weld( w, j, useBias );
			return;
		case P_JOINT_DISTANCE:
			solve_distance( w, j, h, inv_h, useBias );
			return;
		case P_JOINT_PRISMATIC:
			solve_prismatic( w, j, h, inv_h, useBias );
			return;
		case P_JOINT_WHEEL:
			solve_wheel( w, j, h, inv_h, useBias );
			return;
		case P_JOINT_MOTOR:
			solve_motor( w, j, h, inv_h );
			return;
		case P_JOINT_MOUSE:
			solve_mouse( w, j, h );
			return;
		case P_JOINT_FILTER:
			return;
		default:
			break;
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
