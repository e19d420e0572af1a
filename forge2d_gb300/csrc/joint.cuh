// Joint constraints on the device: warm start and solve of the revolute,
// weld and distance joints with the operand order of Box2D v3.1.1's
// revolute_joint.c:195-470, weld_joint.c:142-245 and distance_joint.c:207-420,
// and the softness clamp of joint.c:1346-1352. The type sits in bits 8-10 of
// the joint flags. Joint impulses persist across steps
// in the jimp/jimp2 rows (b2JointSim storage).
#pragma once

#include "dworld.cuh"
#include "kernels.cuh"

#define JF_USED 0x1
#define JF_SPRING 0x2
#define JF_LIMIT 0x4
#define JF_MOTOR 0x8
#define JF_COLLIDE 0x10
#define JF_TYPE_SHIFT 8 // 0 revolute, else the F2D_JOINT_* type
#define JT_WELD 2
#define JT_DISTANCE 3
#define JT_PRISMATIC 4
#define JT_WHEEL 5
#define JT_MOTOR 6
#define JT_MOUSE 7
#define JT_FILTER 8

__device__ __forceinline__ int joint_type( int flags )
{
	return ( flags >> JF_TYPE_SHIFT ) & 0xf;
}

__device__ __forceinline__ float unwind_angle( float r )
{
	return remainderf( r, 2.0f * F2D_PI );
}

template <class BA>
__device__ __forceinline__ void jstate_load( const BA& ba, int i, fv2& v, float& wv, fv2& dp, frot& dq )
{
	BState s = ba.load( i );
	v = mk( s.vx, s.vy );
	wv = s.w;
	dp = mk( s.dpx, s.dpy );
	dq.c = s.dqc;
	dq.s = s.dqs;
}

template <class BA> __device__ __forceinline__ void jstate_store( const BA& ba, int i, fv2 v, float wv )
{
	BState s;
	s.vx = v.x;
	s.vy = v.y;
	s.w = wv;
	s.dpx = s.dpy = 0.0f;
	s.dqc = 1.0f;
	s.dqs = 0.0f;
	ba.store( i, s );
}

template <class BA> __device__ void weld_warm_start( const DWorld& w, const BA& ba, int j );
template <class BA> __device__ void distance_warm_start( const DWorld& w, const BA& ba, int j );
template <class BA> __device__ void prismatic_warm_start( const DWorld& w, const BA& ba, int j );
template <class BA> __device__ void wheel_warm_start( const DWorld& w, const BA& ba, int j );
template <class BA> __device__ void motor_warm_start( const DWorld& w, const BA& ba, int j );
template <class BA> __device__ void mouse_warm_start( const DWorld& w, const BA& ba, int j );
template <class BA> __device__ void weld_solve( const DWorld& w, const BA& ba, int j, bool useBias );
template <class BA>
__device__ void distance_solve( const DWorld& w, const BA& ba, int j, float h, float inv_h, bool useBias );
template <class BA>
__device__ void prismatic_solve( const DWorld& w, const BA& ba, int j, float h, float inv_h, bool useBias );
template <class BA>
__device__ void wheel_solve( const DWorld& w, const BA& ba, int j, float h, float inv_h, bool useBias );
template <class BA> __device__ void motor_solve( const DWorld& w, const BA& ba, int j, float h, float inv_h );
template <class BA> __device__ void mouse_solve( const DWorld& w, const BA& ba, int j, float h );

// revolute_joint.c:261-287; the other types by joint.c:1392-1430
template <class BA> __device__ __forceinline__ void joint_warm_start( const DWorld& w, const BA& ba, int j )
{
	switch ( joint_type( w.jflags[j] ) )
	{
		case JT_WELD:
			weld_warm_start( w, ba, j );
			return;
		case JT_DISTANCE:
			distance_warm_start( w, ba, j );
			return;
		case JT_PRISMATIC:
			prismatic_warm_start( w, ba, j );
			return;
		case JT_WHEEL:
			wheel_warm_start( w, ba, j );
			return;
		case JT_MOTOR:
			motor_warm_start( w, ba, j );
			return;
		case JT_MOUSE:
			mouse_warm_start( w, ba, j );
			return;
		case JT_FILTER:
			return;
		default:
			break;
	}
	int2 idx = w.jindex[j];
	float4 m = w.jprepM[j];
	float mA = m.x, iA = m.y, mB = m.z, iB = m.w;
	float4 p0 = w.jprep0[j];
	float4 imp = __ldcg( w.jimp + j );
	float2 imp2 = __ldcg( w.jimp2 + j );
	fv2 vA, vB, dpA, dpB;
	float wA, wB;
	frot dqA, dqB;
	jstate_load( ba, idx.x, vA, wA, dpA, dqA );
	jstate_load( ba, idx.y, vB, wB, dpB, dqB );
	fv2 rA = rrot( dqA, mk( p0.x, p0.y ) );
	fv2 rB = rrot( dqB, mk( p0.z, p0.w ) );
	fv2 linearImpulse = mk( imp.x, imp.y );
	float axialImpulse = imp.z + imp.w + imp2.x - imp2.y;
	vA = vmulsub( vA, mA, linearImpulse );
	wA -= iA * ( vcross( rA, linearImpulse ) + axialImpulse );
	vB = vmuladd( vB, mB, linearImpulse );
	wB += iB * ( vcross( rB, linearImpulse ) + axialImpulse );
	jstate_store( ba, idx.x, vA, wA );
	jstate_store( ba, idx.y, vB, wB );
}

// revolute_joint.c:289-455
template <class BA>
__device__ __forceinline__ void joint_solve( const DWorld& w, const BA& ba, int j, float h, float inv_h, bool useBias )
{
	int2 idx = w.jindex[j];
	int flags = w.jflags[j];
	switch ( joint_type( flags ) )
	{
		case JT_WELD:
			weld_solve( w, ba, j, useBias );
			return;
		case JT_DISTANCE:
			distance_solve( w, ba, j, h, inv_h, useBias );
			return;
		case JT_PRISMATIC:
			prismatic_solve( w, ba, j, h, inv_h, useBias );
			return;
		case JT_WHEEL:
			wheel_solve( w, ba, j, h, inv_h, useBias );
			return;
		case JT_MOTOR:
			motor_solve( w, ba, j, h, inv_h );
			return;
		case JT_MOUSE:
			mouse_solve( w, ba, j, h );
			return;
		case JT_FILTER:
			return;
		default:
			break;
	}
	float4 m = w.jprepM[j];
	float mA = m.x, iA = m.y, mB = m.z, iB = m.w;
	float4 p0 = w.jprep0[j];
	float4 p1 = w.jprep1[j];
	float4 p2 = w.jprep2[j]; // spring softness biasRate massScale impulseScale, pad
	float4 cs = w.jprep2[w.jointCap + j]; // constraint softness
	float4 d1 = w.jdef1[j]; // referenceAngle targetAngle hertz dampingRatio
	float4 d2 = w.jdef2[j]; // lowerAngle upperAngle maxMotorTorque motorSpeed
	float4 imp = __ldcg( w.jimp + j );
	float2 imp2 = __ldcg( w.jimp2 + j );
	fv2 linearImpulse = mk( imp.x, imp.y );
	float springImpulse = imp.z, motorImpulse = imp.w, lowerImpulse = imp2.x, upperImpulse = imp2.y;
	fv2 vA, vB, dcA, dcB;
	float wA, wB;
	frot dqA, dqB;
	jstate_load( ba, idx.x, vA, wA, dcA, dqA );
	jstate_load( ba, idx.y, vB, wB, dcB, dqB );
	float axialMass = p1.w;
	float deltaAngle = p1.z;
	bool fixedRotation = ( iA + iB == 0.0f );
	if ( ( flags & JF_SPRING ) && fixedRotation == false )
	{
		float jointAngle = relative_angle( dqB, dqA ) + deltaAngle;
		float jointAngleDelta = unwind_angle( jointAngle - d1.y );
		float C = jointAngleDelta;
		float bias = p2.x * C;
		float massScale = p2.y;
		float impulseScale = p2.z;
		float Cdot = wB - wA;
		float impulse = -massScale * axialMass * ( Cdot + bias ) - impulseScale * springImpulse;
		springImpulse += impulse;
		wA -= iA * impulse;
		wB += iB * impulse;
	}
	if ( ( flags & JF_MOTOR ) && fixedRotation == false )
	{
		float Cdot = wB - wA - d2.w;
		float impulse = -axialMass * Cdot;
		float oldImpulse = motorImpulse;
		float maxImpulse = h * d2.z;
		motorImpulse = fclamp_s( motorImpulse + impulse, -maxImpulse, maxImpulse );
		impulse = motorImpulse - oldImpulse;
		wA -= iA * impulse;
		wB += iB * impulse;
	}
	if ( ( flags & JF_LIMIT ) && fixedRotation == false )
	{
		float jointAngle = relative_angle( dqB, dqA ) + deltaAngle - d1.x;
		jointAngle = unwind_angle( jointAngle );
		{
			float C = jointAngle - d2.x;
			float bias = 0.0f, massScale = 1.0f, impulseScale = 0.0f;
			if ( C > 0.0f )
				bias = C * inv_h;
			else if ( useBias )
			{
				bias = cs.x * C;
				massScale = cs.y;
				impulseScale = cs.z;
			}
			float Cdot = wB - wA;
			float oldImpulse = lowerImpulse;
			float impulse = -massScale * axialMass * ( Cdot + bias ) - impulseScale * oldImpulse;
			lowerImpulse = fmax_s( oldImpulse + impulse, 0.0f );
			impulse = lowerImpulse - oldImpulse;
			wA -= iA * impulse;
			wB += iB * impulse;
		}
		{
			float C = d2.y - jointAngle;
			float bias = 0.0f, massScale = 1.0f, impulseScale = 0.0f;
			if ( C > 0.0f )
				bias = C * inv_h;
			else if ( useBias )
			{
				bias = cs.x * C;
				massScale = cs.y;
				impulseScale = cs.z;
			}
			float Cdot = wA - wB;
			float oldImpulse = upperImpulse;
			float impulse = -massScale * axialMass * ( Cdot + bias ) - impulseScale * oldImpulse;
			upperImpulse = fmax_s( oldImpulse + impulse, 0.0f );
			impulse = upperImpulse - oldImpulse;
			wA += iA * impulse;
			wB -= iB * impulse;
		}
	}
	{
		fv2 rA = rrot( dqA, mk( p0.x, p0.y ) );
		fv2 rB = rrot( dqB, mk( p0.z, p0.w ) );
		fv2 Cdot = vsub( vadd( vB, vcrossSV( wB, rB ) ), vadd( vA, vcrossSV( wA, rA ) ) );
		fv2 bias = mk( 0.0f, 0.0f );
		float massScale = 1.0f, impulseScale = 0.0f;
		if ( useBias )
		{
			fv2 separation = vadd( vadd( vsub( dcB, dcA ), vsub( rB, rA ) ), mk( p1.x, p1.y ) );
			bias = vscale( cs.x, separation );
			massScale = cs.y;
			impulseScale = cs.z;
		}
		fv2 Kcx, Kcy;
		Kcx.x = mA + mB + rA.y * rA.y * iA + rB.y * rB.y * iB;
		Kcy.x = -rA.y * rA.x * iA - rB.y * rB.x * iB;
		Kcx.y = Kcy.x;
		Kcy.y = mA + mB + rA.x * rA.x * iA + rB.x * rB.x * iB;
		fv2 b = solve22( Kcx, Kcy, vadd( Cdot, bias ) );
		fv2 impulse;
		impulse.x = -massScale * b.x - impulseScale * linearImpulse.x;
		impulse.y = -massScale * b.y - impulseScale * linearImpulse.y;
		linearImpulse.x += impulse.x;
		linearImpulse.y += impulse.y;
		vA = vmulsub( vA, mA, impulse );
		wA -= iA * vcross( rA, impulse );
		vB = vmuladd( vB, mB, impulse );
		wB += iB * vcross( rB, impulse );
	}
	__stcg( w.jimp + j, make_float4( linearImpulse.x, linearImpulse.y, springImpulse, motorImpulse ) );
	__stcg( w.jimp2 + j, make_float2( lowerImpulse, upperImpulse ) );
	jstate_store( ba, idx.x, vA, wA );
	jstate_store( ba, idx.y, vB, wB );
}

// ---------------------------------------------------------------------------
// weld (weld_joint.c:142-245). Rows: jprep0 anchors, jprep1 deltaCenter
// deltaAngle axialMass, jprep2[j] linear softness, jprep2[cap + j] angular
// softness, jimp linearImpulse.xy angularImpulse.
// ---------------------------------------------------------------------------
template <class BA> __device__ void weld_warm_start( const DWorld& w, const BA& ba, int j )
{
	int2 idx = w.jindex[j];
	float4 m = w.jprepM[j];
	float mA = m.x, iA = m.y, mB = m.z, iB = m.w;
	float4 p0 = w.jprep0[j];
	float4 imp = __ldcg( w.jimp + j );
	fv2 vA, vB, dpA, dpB;
	float wA, wB;
	frot dqA, dqB;
	jstate_load( ba, idx.x, vA, wA, dpA, dqA );
	jstate_load( ba, idx.y, vB, wB, dpB, dqB );
	fv2 rA = rrot( dqA, mk( p0.x, p0.y ) );
	fv2 rB = rrot( dqB, mk( p0.z, p0.w ) );
	fv2 linearImpulse = mk( imp.x, imp.y );
	vA = vmulsub( vA, mA, linearImpulse );
	wA -= iA * ( vcross( rA, linearImpulse ) + imp.z );
	vB = vmuladd( vB, mB, linearImpulse );
	wB += iB * ( vcross( rB, linearImpulse ) + imp.z );
	jstate_store( ba, idx.x, vA, wA );
	jstate_store( ba, idx.y, vB, wB );
}

template <class BA> __device__ void weld_solve( const DWorld& w, const BA& ba, int j, bool useBias )
{
	int2 idx = w.jindex[j];
	float4 m = w.jprepM[j];
	float mA = m.x, iA = m.y, mB = m.z, iB = m.w;
	float4 p0 = w.jprep0[j];
	float4 p1 = w.jprep1[j];
	float4 ls = w.jprep2[j];
	float4 as = w.jprep2[w.jointCap + j];
	float4 d1 = w.jdef1[j]; // referenceAngle linearHertz linearDampingRatio angularHertz
	float4 imp = __ldcg( w.jimp + j );
	fv2 linearImpulse = mk( imp.x, imp.y );
	float angularImpulse = imp.z;
	fv2 vA, vB, dcA, dcB;
	float wA, wB;
	frot dqA, dqB;
	jstate_load( ba, idx.x, vA, wA, dcA, dqA );
	jstate_load( ba, idx.y, vB, wB, dcB, dqB );
	{
		float bias = 0.0f, massScale = 1.0f, impulseScale = 0.0f;
		if ( useBias || d1.w > 0.0f )
		{
			float C = relative_angle( dqB, dqA ) + p1.z;
			bias = as.x * C;
			massScale = as.y;
			impulseScale = as.z;
		}
		float Cdot = wB - wA;
		float impulse = -massScale * p1.w * ( Cdot + bias ) - impulseScale * angularImpulse;
		angularImpulse += impulse;
		wA -= iA * impulse;
		wB += iB * impulse;
	}
	{
		fv2 rA = rrot( dqA, mk( p0.x, p0.y ) );
		fv2 rB = rrot( dqB, mk( p0.z, p0.w ) );
		fv2 bias = mk( 0.0f, 0.0f );
		float massScale = 1.0f, impulseScale = 0.0f;
		if ( useBias || d1.y > 0.0f )
		{
			fv2 C = vadd( vadd( vsub( dcB, dcA ), vsub( rB, rA ) ), mk( p1.x, p1.y ) );
			bias = vscale( ls.x, C );
			massScale = ls.y;
			impulseScale = ls.z;
		}
		fv2 Cdot = vsub( vadd( vB, vcrossSV( wB, rB ) ), vadd( vA, vcrossSV( wA, rA ) ) );
		fv2 Kcx, Kcy;
		Kcx.x = mA + mB + rA.y * rA.y * iA + rB.y * rB.y * iB;
		Kcy.x = -rA.y * rA.x * iA - rB.y * rB.x * iB;
		Kcx.y = Kcy.x;
		Kcy.y = mA + mB + rA.x * rA.x * iA + rB.x * rB.x * iB;
		fv2 b = solve22( Kcx, Kcy, vadd( Cdot, bias ) );
		fv2 impulse;
		impulse.x = -massScale * b.x - impulseScale * linearImpulse.x;
		impulse.y = -massScale * b.y - impulseScale * linearImpulse.y;
		linearImpulse = vadd( linearImpulse, impulse );
		vA = vmulsub( vA, mA, impulse );
		wA -= iA * vcross( rA, impulse );
		vB = vmuladd( vB, mB, impulse );
		wB += iB * vcross( rB, impulse );
	}
	__stcg( w.jimp + j, make_float4( linearImpulse.x, linearImpulse.y, angularImpulse, 0.0f ) );
	jstate_store( ba, idx.x, vA, wA );
	jstate_store( ba, idx.y, vB, wB );
}

// ---------------------------------------------------------------------------
// distance (distance_joint.c:207-420). Rows: jprep0 anchors, jprep1
// deltaCenter . axialMass, jprep2[j] spring softness, jprep2[cap + j]
// constraint softness, jdef1 length minLength maxLength hertz, jdef2
// dampingRatio maxMotorForce motorSpeed, jimp impulse lower upper motor.
// ---------------------------------------------------------------------------
template <class BA> __device__ void distance_warm_start( const DWorld& w, const BA& ba, int j )
{
	int2 idx = w.jindex[j];
	float4 m = w.jprepM[j];
	float mA = m.x, iA = m.y, mB = m.z, iB = m.w;
	float4 p0 = w.jprep0[j];
	float4 p1 = w.jprep1[j];
	float4 imp = __ldcg( w.jimp + j );
	fv2 vA, vB, dpA, dpB;
	float wA, wB;
	frot dqA, dqB;
	jstate_load( ba, idx.x, vA, wA, dpA, dqA );
	jstate_load( ba, idx.y, vB, wB, dpB, dqB );
	fv2 rA = rrot( dqA, mk( p0.x, p0.y ) );
	fv2 rB = rrot( dqB, mk( p0.z, p0.w ) );
	fv2 ds = vadd( vsub( dpB, dpA ), vsub( rB, rA ) );
	fv2 separation = vadd( mk( p1.x, p1.y ), ds );
	fv2 axis = vnormalize( separation );
	float axialImpulse = imp.x + imp.y - imp.z + imp.w;
	fv2 P = vscale( axialImpulse, axis );
	vA = vmulsub( vA, mA, P );
	wA -= iA * vcross( rA, P );
	vB = vmuladd( vB, mB, P );
	wB += iB * vcross( rB, P );
	jstate_store( ba, idx.x, vA, wA );
	jstate_store( ba, idx.y, vB, wB );
}

template <class BA>
__device__ void distance_solve( const DWorld& w, const BA& ba, int j, float h, float inv_h, bool useBias )
{
	int2 idx = w.jindex[j];
	int flags = w.jflags[j];
	float4 m = w.jprepM[j];
	float mA = m.x, iA = m.y, mB = m.z, iB = m.w;
	float4 p0 = w.jprep0[j];
	float4 p1 = w.jprep1[j];
	float4 ds4 = w.jprep2[j];
	float4 cs = w.jprep2[w.jointCap + j];
	float4 d1 = w.jdef1[j];
	float4 d2 = w.jdef2[j];
	float4 imp = __ldcg( w.jimp + j );
	float impulse0 = imp.x, lowerImpulse = imp.y, upperImpulse = imp.z, motorImpulse = imp.w;
	float axialMass = p1.w;
	fv2 vA, vB, dpA, dpB;
	float wA, wB;
	frot dqA, dqB;
	jstate_load( ba, idx.x, vA, wA, dpA, dqA );
	jstate_load( ba, idx.y, vB, wB, dpB, dqB );
	fv2 rA = rrot( dqA, mk( p0.x, p0.y ) );
	fv2 rB = rrot( dqB, mk( p0.z, p0.w ) );
	fv2 ds = vadd( vsub( dpB, dpA ), vsub( rB, rA ) );
	fv2 separation = vadd( mk( p1.x, p1.y ), ds );
	float len = vlen( separation );
	fv2 axis = vnormalize( separation );
	float length = d1.x, minLength = d1.y, maxLength = d1.z, hertz = d1.w;
	if ( ( flags & JF_SPRING ) && ( minLength < maxLength || ( flags & JF_LIMIT ) == 0 ) )
	{
		if ( hertz > 0.0f )
		{
			fv2 vr = vadd( vsub( vB, vA ), vsub( vcrossSV( wB, rB ), vcrossSV( wA, rA ) ) );
			float Cdot = vdot( axis, vr );
			float C = len - length;
			float bias = ds4.x * C;
			float mm = ds4.y * axialMass;
			float impulse = -mm * ( Cdot + bias ) - ds4.z * impulse0;
			impulse0 += impulse;
			fv2 P = vscale( impulse, axis );
			vA = vmulsub( vA, mA, P );
			wA -= iA * vcross( rA, P );
			vB = vmuladd( vB, mB, P );
			wB += iB * vcross( rB, P );
		}
		if ( flags & JF_LIMIT )
		{
			{
				fv2 vr = vadd( vsub( vB, vA ), vsub( vcrossSV( wB, rB ), vcrossSV( wA, rA ) ) );
				float Cdot = vdot( axis, vr );
				float C = len - minLength;
				float bias = 0.0f, massCoeff = 1.0f, impulseCoeff = 0.0f;
				if ( C > 0.0f )
					bias = C * inv_h;
				else if ( useBias )
				{
					bias = cs.x * C;
					massCoeff = cs.y;
					impulseCoeff = cs.z;
				}
				float impulse = -massCoeff * axialMass * ( Cdot + bias ) - impulseCoeff * lowerImpulse;
				float newImpulse = fmax_s( 0.0f, lowerImpulse + impulse );
				impulse = newImpulse - lowerImpulse;
				lowerImpulse = newImpulse;
				fv2 P = vscale( impulse, axis );
				vA = vmulsub( vA, mA, P );
				wA -= iA * vcross( rA, P );
				vB = vmuladd( vB, mB, P );
				wB += iB * vcross( rB, P );
			}
			{
				fv2 vr = vadd( vsub( vA, vB ), vsub( vcrossSV( wA, rA ), vcrossSV( wB, rB ) ) );
				float Cdot = vdot( axis, vr );
				float C = maxLength - len;
				float bias = 0.0f, massScale = 1.0f, impulseScale = 0.0f;
				if ( C > 0.0f )
					bias = C * inv_h;
				else if ( useBias )
				{
					bias = cs.x * C;
					massScale = cs.y;
					impulseScale = cs.z;
				}
				float impulse = -massScale * axialMass * ( Cdot + bias ) - impulseScale * upperImpulse;
				float newImpulse = fmax_s( 0.0f, upperImpulse + impulse );
				impulse = newImpulse - upperImpulse;
				upperImpulse = newImpulse;
				fv2 P = vscale( -impulse, axis );
				vA = vmulsub( vA, mA, P );
				wA -= iA * vcross( rA, P );
				vB = vmuladd( vB, mB, P );
				wB += iB * vcross( rB, P );
			}
		}
		if ( flags & JF_MOTOR )
		{
			fv2 vr = vadd( vsub( vB, vA ), vsub( vcrossSV( wB, rB ), vcrossSV( wA, rA ) ) );
			float Cdot = vdot( axis, vr );
			float impulse = axialMass * ( d2.z - Cdot );
			float oldImpulse = motorImpulse;
			float maxImpulse = h * d2.y;
			motorImpulse = fclamp_s( motorImpulse + impulse, -maxImpulse, maxImpulse );
			impulse = motorImpulse - oldImpulse;
			fv2 P = vscale( impulse, axis );
			vA = vmulsub( vA, mA, P );
			wA -= iA * vcross( rA, P );
			vB = vmuladd( vB, mB, P );
			wB += iB * vcross( rB, P );
		}
	}
	else
	{
		fv2 vr = vadd( vsub( vB, vA ), vsub( vcrossSV( wB, rB ), vcrossSV( wA, rA ) ) );
		float Cdot = vdot( axis, vr );
		float C = len - length;
		float bias = 0.0f, massScale = 1.0f, impulseScale = 0.0f;
		if ( useBias )
		{
			bias = cs.x * C;
			massScale = cs.y;
			impulseScale = cs.z;
		}
		float impulse = -massScale * axialMass * ( Cdot + bias ) - impulseScale * impulse0;
		impulse0 += impulse;
		fv2 P = vscale( impulse, axis );
		vA = vmulsub( vA, mA, P );
		wA -= iA * vcross( rA, P );
		vB = vmuladd( vB, mB, P );
		wB += iB * vcross( rB, P );
	}
	__stcg( w.jimp + j, make_float4( impulse0, lowerImpulse, upperImpulse, motorImpulse ) );
	jstate_store( ba, idx.x, vA, wA );
	jstate_store( ba, idx.y, vB, wB );
}

// ---------------------------------------------------------------------------
// prismatic (prismatic_joint.c:349-604). Rows: jdef1 localAxisA.xy
// referenceAngle targetTranslation, jdef2 lower upper maxMotorForce
// motorSpeed, jimp impulse.xy (perpendicular, angular) spring motor, jimp2
// lower upper, jprep1 deltaCenter deltaAngle axialMass, jprep2[j] spring
// softness, jprep2[cap + j] constraint softness, jprep3 axisA.xy.
// ---------------------------------------------------------------------------
template <class BA> __device__ void prismatic_warm_start( const DWorld& w, const BA& ba, int j )
{
	int2 idx = w.jindex[j];
	float4 m = w.jprepM[j];
	float mA = m.x, iA = m.y, mB = m.z, iB = m.w;
	float4 p0 = w.jprep0[j];
	float4 p1 = w.jprep1[j];
	float4 p3 = w.jprep3[j];
	float4 imp = __ldcg( w.jimp + j );
	float2 imp2 = __ldcg( w.jimp2 + j );
	fv2 vA, vB, dpA, dpB;
	float wA, wB;
	frot dqA, dqB;
	jstate_load( ba, idx.x, vA, wA, dpA, dqA );
	jstate_load( ba, idx.y, vB, wB, dpB, dqB );
	fv2 rA = rrot( dqA, mk( p0.x, p0.y ) );
	fv2 rB = rrot( dqB, mk( p0.z, p0.w ) );
	fv2 d = vadd( vadd( vsub( dpB, dpA ), mk( p1.x, p1.y ) ), vsub( rB, rA ) );
	fv2 axisA = rrot( dqA, mk( p3.x, p3.y ) );
	float a1 = vcross( vadd( d, rA ), axisA );
	float a2 = vcross( rB, axisA );
	float axialImpulse = imp.z + imp.w + imp2.x - imp2.y;
	fv2 perpA = vleft( axisA );
	float s1 = vcross( vadd( d, rA ), perpA );
	float s2 = vcross( rB, perpA );
	float perpImpulse = imp.x;
	float angleImpulse = imp.y;
	fv2 P = vadd( vscale( axialImpulse, axisA ), vscale( perpImpulse, perpA ) );
	float LA = axialImpulse * a1 + perpImpulse * s1 + angleImpulse;
	float LB = axialImpulse * a2 + perpImpulse * s2 + angleImpulse;
	vA = vmulsub( vA, mA, P );
	wA -= iA * LA;
	vB = vmuladd( vB, mB, P );
	wB += iB * LB;
	jstate_store( ba, idx.x, vA, wA );
	jstate_store( ba, idx.y, vB, wB );
}

template <class BA>
__device__ void prismatic_solve( const DWorld& w, const BA& ba, int j, float h, float inv_h, bool useBias )
{
	int2 idx = w.jindex[j];
	int flags = w.jflags[j];
	float4 m = w.jprepM[j];
	float mA = m.x, iA = m.y, mB = m.z, iB = m.w;
	float4 p0 = w.jprep0[j];
	float4 p1 = w.jprep1[j];
	float4 p3 = w.jprep3[j];
	float4 sp = w.jprep2[j];
	float4 cs = w.jprep2[w.jointCap + j];
	float4 d1 = w.jdef1[j];
	float4 d2 = w.jdef2[j];
	float4 imp = __ldcg( w.jimp + j );
	float2 imp2 = __ldcg( w.jimp2 + j );
	fv2 impulse2 = mk( imp.x, imp.y );
	float springImpulse = imp.z, motorImpulse = imp.w, lowerImpulse = imp2.x, upperImpulse = imp2.y;
	float axialMass = p1.w;
	fv2 vA, vB, dpA, dpB;
	float wA, wB;
	frot dqA, dqB;
	jstate_load( ba, idx.x, vA, wA, dpA, dqA );
	jstate_load( ba, idx.y, vB, wB, dpB, dqB );
	fv2 rA = rrot( dqA, mk( p0.x, p0.y ) );
	fv2 rB = rrot( dqB, mk( p0.z, p0.w ) );
	fv2 d = vadd( vadd( vsub( dpB, dpA ), mk( p1.x, p1.y ) ), vsub( rB, rA ) );
	fv2 axisA = rrot( dqA, mk( p3.x, p3.y ) );
	float translation = vdot( axisA, d );
	float a1 = vcross( vadd( d, rA ), axisA );
	float a2 = vcross( rB, axisA );
	if ( flags & JF_SPRING )
	{
		float C = translation - d1.w;
		float bias = sp.x * C;
		float massScale = sp.y;
		float impulseScale = sp.z;
		float Cdot = vdot( axisA, vsub( vB, vA ) ) + a2 * wB - a1 * wA;
		float deltaImpulse = -massScale * axialMass * ( Cdot + bias ) - impulseScale * springImpulse;
		springImpulse += deltaImpulse;
		fv2 P = vscale( deltaImpulse, axisA );
		float LA = deltaImpulse * a1;
		float LB = deltaImpulse * a2;
		vA = vmulsub( vA, mA, P );
		wA -= iA * LA;
		vB = vmuladd( vB, mB, P );
		wB += iB * LB;
	}
	if ( flags & JF_MOTOR )
	{
		float Cdot = vdot( axisA, vsub( vB, vA ) ) + a2 * wB - a1 * wA;
		float impulse = axialMass * ( d2.w - Cdot );
		float oldImpulse = motorImpulse;
		float maxImpulse = h * d2.z;
		motorImpulse = fclamp_s( motorImpulse + impulse, -maxImpulse, maxImpulse );
		impulse = motorImpulse - oldImpulse;
		fv2 P = vscale( impulse, axisA );
		float LA = impulse * a1;
		float LB = impulse * a2;
		vA = vmulsub( vA, mA, P );
		wA -= iA * LA;
		vB = vmuladd( vB, mB, P );
		wB += iB * LB;
	}
	if ( flags & JF_LIMIT )
	{
		{
			float C = translation - d2.x;
			float bias = 0.0f, massScale = 1.0f, impulseScale = 0.0f;
			if ( C > 0.0f )
				bias = C * inv_h;
			else if ( useBias )
			{
				bias = cs.x * C;
				massScale = cs.y;
				impulseScale = cs.z;
			}
			float oldImpulse = lowerImpulse;
			float Cdot = vdot( axisA, vsub( vB, vA ) ) + a2 * wB - a1 * wA;
			float impulse = -axialMass * massScale * ( Cdot + bias ) - impulseScale * oldImpulse;
			lowerImpulse = fmax_s( oldImpulse + impulse, 0.0f );
			impulse = lowerImpulse - oldImpulse;
			fv2 P = vscale( impulse, axisA );
			float LA = impulse * a1;
			float LB = impulse * a2;
			vA = vmulsub( vA, mA, P );
			wA -= iA * LA;
			vB = vmuladd( vB, mB, P );
			wB += iB * LB;
		}
		{
			float C = d2.y - translation;
			float bias = 0.0f, massScale = 1.0f, impulseScale = 0.0f;
			if ( C > 0.0f )
				bias = C * inv_h;
			else if ( useBias )
			{
				bias = cs.x * C;
				massScale = cs.y;
				impulseScale = cs.z;
			}
			float oldImpulse = upperImpulse;
			float Cdot = vdot( axisA, vsub( vA, vB ) ) + a1 * wA - a2 * wB;
			float impulse = -axialMass * massScale * ( Cdot + bias ) - impulseScale * oldImpulse;
			upperImpulse = fmax_s( oldImpulse + impulse, 0.0f );
			impulse = upperImpulse - oldImpulse;
			fv2 P = vscale( impulse, axisA );
			float LA = impulse * a1;
			float LB = impulse * a2;
			vA = vmuladd( vA, mA, P );
			wA += iA * LA;
			vB = vmulsub( vB, mB, P );
			wB -= iB * LB;
		}
	}
	{
		fv2 perpA = vleft( axisA );
		float s1 = vcross( vadd( d, rA ), perpA );
		float s2 = vcross( rB, perpA );
		fv2 Cdot;
		Cdot.x = vdot( perpA, vsub( vB, vA ) ) + s2 * wB - s1 * wA;
		Cdot.y = wB - wA;
		fv2 bias = mk( 0.0f, 0.0f );
		float massScale = 1.0f, impulseScale = 0.0f;
		if ( useBias )
		{
			fv2 C;
			C.x = vdot( perpA, d );
			C.y = relative_angle( dqB, dqA ) + p1.z;
			bias = vscale( cs.x, C );
			massScale = cs.y;
			impulseScale = cs.z;
		}
		float k11 = mA + mB + iA * s1 * s1 + iB * s2 * s2;
		float k12 = iA * s1 + iB * s2;
		float k22 = iA + iB;
		if ( k22 == 0.0f )
			k22 = 1.0f;
		fv2 b = solve22( mk( k11, k12 ), mk( k12, k22 ), vadd( Cdot, bias ) );
		fv2 impulse;
		impulse.x = -massScale * b.x - impulseScale * impulse2.x;
		impulse.y = -massScale * b.y - impulseScale * impulse2.y;
		impulse2.x += impulse.x;
		impulse2.y += impulse.y;
		fv2 P = vscale( impulse.x, perpA );
		float LA = impulse.x * s1 + impulse.y;
		float LB = impulse.x * s2 + impulse.y;
		vA = vmulsub( vA, mA, P );
		wA -= iA * LA;
		vB = vmuladd( vB, mB, P );
		wB += iB * LB;
	}
	__stcg( w.jimp + j, make_float4( impulse2.x, impulse2.y, springImpulse, motorImpulse ) );
	__stcg( w.jimp2 + j, make_float2( lowerImpulse, upperImpulse ) );
	jstate_store( ba, idx.x, vA, wA );
	jstate_store( ba, idx.y, vB, wB );
}

// ---------------------------------------------------------------------------
// wheel (wheel_joint.c:265-488). Rows: jdef1 localAxisA.xy hertz
// dampingRatio, jdef2 lower upper maxMotorTorque motorSpeed, jimp perp spring
// motor, jimp2 lower upper, jprep1 deltaCenter perpMass axialMass, jprep2[j]
// spring softness, jprep2[cap + j] constraint softness, jprep3 axisA.xy
// motorMass.
// ---------------------------------------------------------------------------
template <class BA> __device__ void wheel_warm_start( const DWorld& w, const BA& ba, int j )
{
	int2 idx = w.jindex[j];
	float4 m = w.jprepM[j];
	float mA = m.x, iA = m.y, mB = m.z, iB = m.w;
	float4 p0 = w.jprep0[j];
	float4 p1 = w.jprep1[j];
	float4 p3 = w.jprep3[j];
	float4 imp = __ldcg( w.jimp + j );
	float2 imp2 = __ldcg( w.jimp2 + j );
	fv2 vA, vB, dpA, dpB;
	float wA, wB;
	frot dqA, dqB;
	jstate_load( ba, idx.x, vA, wA, dpA, dqA );
	jstate_load( ba, idx.y, vB, wB, dpB, dqB );
	fv2 rA = rrot( dqA, mk( p0.x, p0.y ) );
	fv2 rB = rrot( dqB, mk( p0.z, p0.w ) );
	fv2 d = vadd( vadd( vsub( dpB, dpA ), mk( p1.x, p1.y ) ), vsub( rB, rA ) );
	fv2 axisA = rrot( dqA, mk( p3.x, p3.y ) );
	fv2 perpA = vleft( axisA );
	float a1 = vcross( vadd( d, rA ), axisA );
	float a2 = vcross( rB, axisA );
	float s1 = vcross( vadd( d, rA ), perpA );
	float s2 = vcross( rB, perpA );
	float axialImpulse = imp.y + imp2.x - imp2.y;
	fv2 P = vadd( vscale( axialImpulse, axisA ), vscale( imp.x, perpA ) );
	float LA = axialImpulse * a1 + imp.x * s1 + imp.z;
	float LB = axialImpulse * a2 + imp.x * s2 + imp.z;
	vA = vmulsub( vA, mA, P );
	wA -= iA * LA;
	vB = vmuladd( vB, mB, P );
	wB += iB * LB;
	jstate_store( ba, idx.x, vA, wA );
	jstate_store( ba, idx.y, vB, wB );
}

template <class BA>
__device__ void wheel_solve( const DWorld& w, const BA& ba, int j, float h, float inv_h, bool useBias )
{
	int2 idx = w.jindex[j];
	int flags = w.jflags[j];
	float4 m = w.jprepM[j];
	float mA = m.x, iA = m.y, mB = m.z, iB = m.w;
	float4 p0 = w.jprep0[j];
	float4 p1 = w.jprep1[j];
	float4 p3 = w.jprep3[j];
	float4 sp = w.jprep2[j];
	float4 cs = w.jprep2[w.jointCap + j];
	float4 d2 = w.jdef2[j];
	float4 imp = __ldcg( w.jimp + j );
	float2 imp2 = __ldcg( w.jimp2 + j );
	float perpImpulse = imp.x, springImpulse = imp.y, motorImpulse = imp.z;
	float lowerImpulse = imp2.x, upperImpulse = imp2.y;
	float perpMass = p1.z, axialMass = p1.w, motorMass = p3.z;
	fv2 vA, vB, dpA, dpB;
	float wA, wB;
	frot dqA, dqB;
	jstate_load( ba, idx.x, vA, wA, dpA, dqA );
	jstate_load( ba, idx.y, vB, wB, dpB, dqB );
	bool fixedRotation = ( iA + iB == 0.0f );
	fv2 rA = rrot( dqA, mk( p0.x, p0.y ) );
	fv2 rB = rrot( dqB, mk( p0.z, p0.w ) );
	fv2 d = vadd( vadd( vsub( dpB, dpA ), mk( p1.x, p1.y ) ), vsub( rB, rA ) );
	fv2 axisA = rrot( dqA, mk( p3.x, p3.y ) );
	float translation = vdot( axisA, d );
	float a1 = vcross( vadd( d, rA ), axisA );
	float a2 = vcross( rB, axisA );
	if ( ( flags & JF_MOTOR ) && fixedRotation == false )
	{
		float Cdot = wB - wA - d2.w;
		float impulse = -motorMass * Cdot;
		float oldImpulse = motorImpulse;
		float maxImpulse = h * d2.z;
		motorImpulse = fclamp_s( motorImpulse + impulse, -maxImpulse, maxImpulse );
		impulse = motorImpulse - oldImpulse;
		wA -= iA * impulse;
		wB += iB * impulse;
	}
	if ( flags & JF_SPRING )
	{
		float C = translation;
		float bias = sp.x * C;
		float massScale = sp.y;
		float impulseScale = sp.z;
		float Cdot = vdot( axisA, vsub( vB, vA ) ) + a2 * wB - a1 * wA;
		float impulse = -massScale * axialMass * ( Cdot + bias ) - impulseScale * springImpulse;
		springImpulse += impulse;
		fv2 P = vscale( impulse, axisA );
		float LA = impulse * a1;
		float LB = impulse * a2;
		vA = vmulsub( vA, mA, P );
		wA -= iA * LA;
		vB = vmuladd( vB, mB, P );
		wB += iB * LB;
	}
	if ( flags & JF_LIMIT )
	{
		{
			float C = translation - d2.x;
			float bias = 0.0f, massScale = 1.0f, impulseScale = 0.0f;
			if ( C > 0.0f )
				bias = C * inv_h;
			else if ( useBias )
			{
				bias = cs.x * C;
				massScale = cs.y;
				impulseScale = cs.z;
			}
			float Cdot = vdot( axisA, vsub( vB, vA ) ) + a2 * wB - a1 * wA;
			float impulse = -massScale * axialMass * ( Cdot + bias ) - impulseScale * lowerImpulse;
			float oldImpulse = lowerImpulse;
			lowerImpulse = fmax_s( oldImpulse + impulse, 0.0f );
			impulse = lowerImpulse - oldImpulse;
			fv2 P = vscale( impulse, axisA );
			float LA = impulse * a1;
			float LB = impulse * a2;
			vA = vmulsub( vA, mA, P );
			wA -= iA * LA;
			vB = vmuladd( vB, mB, P );
			wB += iB * LB;
		}
		{
			float C = d2.y - translation;
			float bias = 0.0f, massScale = 1.0f, impulseScale = 0.0f;
			if ( C > 0.0f )
				bias = C * inv_h;
			else if ( useBias )
			{
				bias = cs.x * C;
				massScale = cs.y;
				impulseScale = cs.z;
			}
			float Cdot = vdot( axisA, vsub( vA, vB ) ) + a1 * wA - a2 * wB;
			float impulse = -massScale * axialMass * ( Cdot + bias ) - impulseScale * upperImpulse;
			float oldImpulse = upperImpulse;
			upperImpulse = fmax_s( oldImpulse + impulse, 0.0f );
			impulse = upperImpulse - oldImpulse;
			fv2 P = vscale( impulse, axisA );
			float LA = impulse * a1;
			float LB = impulse * a2;
			vA = vmuladd( vA, mA, P );
			wA += iA * LA;
			vB = vmulsub( vB, mB, P );
			wB -= iB * LB;
		}
	}
	{
		fv2 perpA = vleft( axisA );
		float bias = 0.0f, massScale = 1.0f, impulseScale = 0.0f;
		if ( useBias )
		{
			float C = vdot( perpA, d );
			bias = cs.x * C;
			massScale = cs.y;
			impulseScale = cs.z;
		}
		float s1 = vcross( vadd( d, rA ), perpA );
		float s2 = vcross( rB, perpA );
		float Cdot = vdot( perpA, vsub( vB, vA ) ) + s2 * wB - s1 * wA;
		float impulse = -massScale * perpMass * ( Cdot + bias ) - impulseScale * perpImpulse;
		perpImpulse += impulse;
		fv2 P = vscale( impulse, perpA );
		float LA = impulse * s1;
		float LB = impulse * s2;
		vA = vmulsub( vA, mA, P );
		wA -= iA * LA;
		vB = vmuladd( vB, mB, P );
		wB += iB * LB;
	}
	__stcg( w.jimp + j, make_float4( perpImpulse, springImpulse, motorImpulse, 0.0f ) );
	__stcg( w.jimp2 + j, make_float2( lowerImpulse, upperImpulse ) );
	jstate_store( ba, idx.x, vA, wA );
	jstate_store( ba, idx.y, vB, wB );
}

// ---------------------------------------------------------------------------
// motor (motor_joint.c:162-262). Rows: jdef1 linearOffset.xy angularOffset
// maxForce, jdef2 maxTorque correctionFactor, jimp linearImpulse.xy
// angularImpulse, jprep1 deltaCenter deltaAngle angularMass, jprep3 the
// inverse 2x2 linear mass (columns cx, cy).
// ---------------------------------------------------------------------------
template <class BA> __device__ void motor_warm_start( const DWorld& w, const BA& ba, int j )
{
	weld_warm_start( w, ba, j ); // same operands: linearImpulse.xy, angularImpulse
}

template <class BA> __device__ void motor_solve( const DWorld& w, const BA& ba, int j, float h, float inv_h )
{
	int2 idx = w.jindex[j];
	float4 m = w.jprepM[j];
	float mA = m.x, iA = m.y, mB = m.z, iB = m.w;
	float4 p0 = w.jprep0[j];
	float4 p1 = w.jprep1[j];
	float4 p3 = w.jprep3[j];
	float4 d1 = w.jdef1[j];
	float4 d2 = w.jdef2[j];
	float4 imp = __ldcg( w.jimp + j );
	fv2 linearImpulse = mk( imp.x, imp.y );
	float angularImpulse = imp.z;
	float correctionFactor = d2.y;
	fv2 vA, vB, dpA, dpB;
	float wA, wB;
	frot dqA, dqB;
	jstate_load( ba, idx.x, vA, wA, dpA, dqA );
	jstate_load( ba, idx.y, vB, wB, dpB, dqB );
	{
		float angularSeparation = relative_angle( dqB, dqA ) + p1.z;
		angularSeparation = unwind_angle( angularSeparation );
		float angularBias = inv_h * correctionFactor * angularSeparation;
		float Cdot = wB - wA;
		float impulse = -p1.w * ( Cdot + angularBias );
		float oldImpulse = angularImpulse;
		float maxImpulse = h * d2.x;
		angularImpulse = fclamp_s( angularImpulse + impulse, -maxImpulse, maxImpulse );
		impulse = angularImpulse - oldImpulse;
		wA -= iA * impulse;
		wB += iB * impulse;
	}
	{
		fv2 rA = rrot( dqA, mk( p0.x, p0.y ) );
		fv2 rB = rrot( dqB, mk( p0.z, p0.w ) );
		fv2 ds = vadd( vsub( dpB, dpA ), vsub( rB, rA ) );
		fv2 linearSeparation = vadd( mk( p1.x, p1.y ), ds );
		fv2 linearBias = vscale( inv_h * correctionFactor, linearSeparation );
		fv2 Cdot = vsub( vadd( vB, vcrossSV( wB, rB ) ), vadd( vA, vcrossSV( wA, rA ) ) );
		fv2 b = mulMV( mk( p3.x, p3.y ), mk( p3.z, p3.w ), vadd( Cdot, linearBias ) );
		fv2 impulse = mk( -b.x, -b.y );
		fv2 oldImpulse = linearImpulse;
		float maxImpulse = h * d1.w;
		linearImpulse = vadd( linearImpulse, impulse );
		if ( vlen2( linearImpulse ) > maxImpulse * maxImpulse )
		{
			linearImpulse = vnormalize( linearImpulse );
			linearImpulse.x *= maxImpulse;
			linearImpulse.y *= maxImpulse;
		}
		impulse = vsub( linearImpulse, oldImpulse );
		vA = vmulsub( vA, mA, impulse );
		wA -= iA * vcross( rA, impulse );
		vB = vmuladd( vB, mB, impulse );
		wB += iB * vcross( rB, impulse );
	}
	__stcg( w.jimp + j, make_float4( linearImpulse.x, linearImpulse.y, angularImpulse, 0.0f ) );
	jstate_store( ba, idx.x, vA, wA );
	jstate_store( ba, idx.y, vB, wB );
}

// ---------------------------------------------------------------------------
// mouse (mouse_joint.c:130-214): body B only. Rows: jdef1 target.xy hertz
// dampingRatio, jdef2 maxForce, jimp linearImpulse.xy angularImpulse, jprep1
// deltaCenter, jprep2[j] linear softness, jprep2[cap + j] angular softness,
// jprep3 the inverse 2x2 linear mass. A static body B (which the reference
// does not allow) is left alone.
// ---------------------------------------------------------------------------
template <class BA> __device__ void mouse_warm_start( const DWorld& w, const BA& ba, int j )
{
	int2 idx = w.jindex[j];
	if ( idx.y < 0 )
		return;
	float4 m = w.jprepM[j];
	float mB = m.z, iB = m.w;
	float4 p0 = w.jprep0[j];
	float4 imp = __ldcg( w.jimp + j );
	fv2 vB, dpB;
	float wB;
	frot dqB;
	jstate_load( ba, idx.y, vB, wB, dpB, dqB );
	fv2 rB = rrot( dqB, mk( p0.z, p0.w ) );
	fv2 linearImpulse = mk( imp.x, imp.y );
	vB = vmuladd( vB, mB, linearImpulse );
	wB += iB * ( vcross( rB, linearImpulse ) + imp.z );
	jstate_store( ba, idx.y, vB, wB );
}

template <class BA> __device__ void mouse_solve( const DWorld& w, const BA& ba, int j, float h )
{
	int2 idx = w.jindex[j];
	if ( idx.y < 0 )
		return;
	float4 m = w.jprepM[j];
	float mB = m.z, iB = m.w;
	float4 p0 = w.jprep0[j];
	float4 p1 = w.jprep1[j];
	float4 p3 = w.jprep3[j];
	float4 ls = w.jprep2[j];
	float4 as = w.jprep2[w.jointCap + j];
	float4 d2 = w.jdef2[j];
	float4 imp = __ldcg( w.jimp + j );
	fv2 linearImpulse = mk( imp.x, imp.y );
	float angularImpulse = imp.z;
	fv2 vB, dpB;
	float wB;
	frot dqB;
	jstate_load( ba, idx.y, vB, wB, dpB, dqB );
	{
		float massScale = as.y;
		float impulseScale = as.z;
		float impulse = iB > 0.0f ? -wB / iB : 0.0f;
		impulse = massScale * impulse - impulseScale * angularImpulse;
		angularImpulse += impulse;
		wB += iB * impulse;
	}
	float maxImpulse = d2.x * h;
	{
		fv2 rB = rrot( dqB, mk( p0.z, p0.w ) );
		fv2 Cdot = vadd( vB, vcrossSV( wB, rB ) );
		fv2 separation = vadd( vadd( dpB, rB ), mk( p1.x, p1.y ) );
		fv2 bias = vscale( ls.x, separation );
		float massScale = ls.y;
		float impulseScale = ls.z;
		fv2 b = mulMV( mk( p3.x, p3.y ), mk( p3.z, p3.w ), vadd( Cdot, bias ) );
		fv2 impulse;
		impulse.x = -massScale * b.x - impulseScale * linearImpulse.x;
		impulse.y = -massScale * b.y - impulseScale * linearImpulse.y;
		fv2 oldImpulse = linearImpulse;
		linearImpulse.x += impulse.x;
		linearImpulse.y += impulse.y;
		float mag = vlen( linearImpulse );
		if ( mag > maxImpulse )
			linearImpulse = vscale( maxImpulse, vnormalize( linearImpulse ) );
		impulse.x = linearImpulse.x - oldImpulse.x;
		impulse.y = linearImpulse.y - oldImpulse.y;
		vB = vmuladd( vB, mB, impulse );
		wB += iB * vcross( rB, impulse );
	}
	__stcg( w.jimp + j, make_float4( linearImpulse.x, linearImpulse.y, angularImpulse, 0.0f ) );
	jstate_store( ba, idx.y, vB, wB );
}

void launch_prepare_joints( DWorld& w, StepScratch& s, cudaStream_t st, float h, float inv_h, Soft jointSoft );
