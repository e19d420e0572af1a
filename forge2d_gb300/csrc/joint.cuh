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
#define JF_TYPE_SHIFT 8 // 0 revolute, 2 weld, 3 distance
#define JT_WELD 2
#define JT_DISTANCE 3

__device__ __forceinline__ int joint_type( int flags )
{
	return ( flags >> JF_TYPE_SHIFT ) & 7;
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
template <class BA> __device__ void weld_solve( const DWorld& w, const BA& ba, int j, bool useBias );
template <class BA>
__device__ void distance_solve( const DWorld& w, const BA& ba, int j, float h, float inv_h, bool useBias );

// revolute_joint.c:261-287
template <class BA> __device__ __forceinline__ void joint_warm_start( const DWorld& w, const BA& ba, int j )
{
	int type = joint_type( w.jflags[j] );
	if ( type == JT_WELD )
	{
		weld_warm_start( w, ba, j );
		return;
	}
	if ( type == JT_DISTANCE )
	{
		distance_warm_start( w, ba, j );
		return;
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
	if ( joint_type( flags ) == JT_WELD )
	{
		weld_solve( w, ba, j, useBias );
		return;
	}
	if ( joint_type( flags ) == JT_DISTANCE )
	{
		distance_solve( w, ba, j, h, inv_h, useBias );
		return;
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

void launch_prepare_joints( DWorld& w, StepScratch& s, cudaStream_t st, float h, float inv_h, Soft jointSoft );
