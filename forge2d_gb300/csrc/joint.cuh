// Revolute joint constraint on the device: prepare, warm start and solve with
// the operand order of Box2D v3.1.1's revolute_joint.c:195-470 and the
// softness clamp of joint.c:1346-1352. Joint impulses persist across steps
// in the jimp/jimp2 rows (b2JointSim storage).
#pragma once

#include "dworld.cuh"
#include "kernels.cuh"

#define JF_USED 0x1
#define JF_SPRING 0x2
#define JF_LIMIT 0x4
#define JF_MOTOR 0x8
#define JF_COLLIDE 0x10

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

// revolute_joint.c:261-287
template <class BA> __device__ __forceinline__ void joint_warm_start( const DWorld& w, const BA& ba, int j )
{
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

void launch_prepare_joints( DWorld& w, StepScratch& s, cudaStream_t st, float h, float inv_h, Soft jointSoft );
