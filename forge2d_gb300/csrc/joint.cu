// Joint preparation and the per-colour joint slot lists of the solver.
// Reference: packages/forge2d/third_party/box2d/src/joint.c:1346-1390
// (softness clamp, type dispatch), revolute_joint.c:195-259,
// weld_joint.c:83-140, distance_joint.c:158-205, prismatic_joint.c:279-346,
// wheel_joint.c:183-262, motor_joint.c:99-160, mouse_joint.c:77-128.
#include "joint.cuh"

__global__ void k_prepare_joints( DWorld w, float h, float inv_h, Soft jointSoft )
{
	int n = w.jointCount;
	for ( int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x )
	{
		// joints outside the graph (sleeping sets) are not solved
		if ( ( w.jflags[j] & JF_USED ) == 0 || w.jcolor[j] == F2D_NULL )
			continue;
		int2 jb = w.jbody[j];
		int a = jb.x, b = jb.y;
		int fa = w.bflags[a], fb = w.bflags[b];
		float4 ma = w.massv[a], mb = w.massv[b];
		float mA = ma.x, iA = ma.y, mB = mb.x, iB = mb.y;
		w.jprepM[j] = make_float4( mA, iA, mB, iB );
		w.jindex[j] = make_int2( body_type( fa ) == 0 ? -1 : a, body_type( fb ) == 0 ? -1 : b );
		float4 xa = w.xf[a], xb = w.xf[b];
		frot qA, qB;
		qA.c = xa.z;
		qA.s = xa.w;
		qB.c = xb.z;
		qB.s = xb.w;
		float4 d0 = w.jdef0[j];
		float2 lca = w.localCenter[a], lcb = w.localCenter[b];
		fv2 anchorA = rrot( qA, vsub( mk( d0.x, d0.y ), mk( lca.x, lca.y ) ) );
		fv2 anchorB = rrot( qB, vsub( mk( d0.z, d0.w ), mk( lcb.x, lcb.y ) ) );
		float2 ca = w.center[a], cb = w.center[b];
		fv2 deltaCenter = vsub( mk( cb.x, cb.y ), mk( ca.x, ca.y ) );
		int type = joint_type( w.jflags[j] );
		if ( type == JT_WELD )
		{
			// weld_joint.c:116-140
			float4 d1 = w.jdef1[j]; // referenceAngle linearHertz linearDampingRatio angularHertz
			float4 d2 = w.jdef2[j]; // angularDampingRatio
			float deltaAngle = unwind_angle( relative_angle( qB, qA ) - d1.x );
			float k = iA + iB;
			float axialMass = k > 0.0f ? 1.0f / k : 0.0f;
			Soft ls = d1.y == 0.0f ? jointSoft : make_soft( d1.y, d1.z, h );
			Soft as = d1.w == 0.0f ? jointSoft : make_soft( d1.w, d2.x, h );
			w.jprep0[j] = make_float4( anchorA.x, anchorA.y, anchorB.x, anchorB.y );
			w.jprep1[j] = make_float4( deltaCenter.x, deltaCenter.y, deltaAngle, axialMass );
			w.jprep2[j] = make_float4( ls.biasRate, ls.massScale, ls.impulseScale, 0.0f );
			w.jprep2[w.jointCap + j] = make_float4( as.biasRate, as.massScale, as.impulseScale, 0.0f );
			if ( w.enableWarmStarting == 0 )
				w.jimp[j] = make_float4( 0.0f, 0.0f, 0.0f, 0.0f );
			continue;
		}
		if ( type == JT_PRISMATIC || type == JT_WHEEL )
		{
			// prismatic_joint.c:316-346, wheel_joint.c:220-262
			float4 d1 = w.jdef1[j];
			fv2 axisA = rrot( qA, mk( d1.x, d1.y ) );
			fv2 rA = anchorA, rB = anchorB;
			fv2 d = vadd( deltaCenter, vsub( rB, rA ) );
			float a1 = vcross( vadd( d, rA ), axisA );
			float a2 = vcross( rB, axisA );
			w.jprep0[j] = make_float4( anchorA.x, anchorA.y, anchorB.x, anchorB.y );
			w.jprep2[w.jointCap + j] =
				make_float4( jointSoft.biasRate, jointSoft.massScale, jointSoft.impulseScale, 0.0f );
			if ( type == JT_PRISMATIC )
			{
				float deltaAngle = unwind_angle( relative_angle( qB, qA ) - d1.z );
				float k = mA + mB + iA * a1 * a1 + iB * a2 * a2;
				float axialMass = k > 0.0f ? 1.0f / k : 0.0f;
				float4 d3 = w.jdef3[j];
				Soft sp = make_soft( d3.x, d3.y, h );
				w.jprep1[j] = make_float4( deltaCenter.x, deltaCenter.y, deltaAngle, axialMass );
				w.jprep2[j] = make_float4( sp.biasRate, sp.massScale, sp.impulseScale, 0.0f );
				w.jprep3[j] = make_float4( axisA.x, axisA.y, 0.0f, 0.0f );
			}
			else
			{
				fv2 perpA = vleft( axisA );
				float s1 = vcross( vadd( d, rA ), perpA );
				float s2 = vcross( rB, perpA );
				float kp = mA + mB + iA * s1 * s1 + iB * s2 * s2;
				float perpMass = kp > 0.0f ? 1.0f / kp : 0.0f;
				float ka = mA + mB + iA * a1 * a1 + iB * a2 * a2;
				float axialMass = ka > 0.0f ? 1.0f / ka : 0.0f;
				Soft sp = make_soft( d1.z, d1.w, h );
				float km = iA + iB;
				float motorMass = km > 0.0f ? 1.0f / km : 0.0f;
				w.jprep1[j] = make_float4( deltaCenter.x, deltaCenter.y, perpMass, axialMass );
				w.jprep2[j] = make_float4( sp.biasRate, sp.massScale, sp.impulseScale, 0.0f );
				w.jprep3[j] = make_float4( axisA.x, axisA.y, motorMass, 0.0f );
			}
			if ( w.enableWarmStarting == 0 )
			{
				w.jimp[j] = make_float4( 0.0f, 0.0f, 0.0f, 0.0f );
				w.jimp2[j] = make_float2( 0.0f, 0.0f );
			}
			continue;
		}
		if ( type == JT_MOTOR )
		{
			// motor_joint.c:138-160
			float4 d1 = w.jdef1[j]; // linearOffset.xy angularOffset maxForce
			fv2 dc = vsub( deltaCenter, mk( d1.x, d1.y ) );
			float deltaAngle = relative_angle( qB, qA ) - d1.z;
			fv2 rA = anchorA, rB = anchorB;
			fv2 cx, cy;
			cx.x = mA + mB + rA.y * rA.y * iA + rB.y * rB.y * iB;
			cx.y = -rA.y * rA.x * iA - rB.y * rB.x * iB;
			cy.x = cx.y;
			cy.y = mA + mB + rA.x * rA.x * iA + rB.x * rB.x * iB;
			float ka = iA + iB;
			float angularMass = ka > 0.0f ? 1.0f / ka : 0.0f;
			w.jprep0[j] = make_float4( anchorA.x, anchorA.y, anchorB.x, anchorB.y );
			w.jprep1[j] = make_float4( dc.x, dc.y, deltaAngle, angularMass );
			w.jprep3[j] = inverse22( cx, cy );
			if ( w.enableWarmStarting == 0 )
				w.jimp[j] = make_float4( 0.0f, 0.0f, 0.0f, 0.0f );
			continue;
		}
		if ( type == JT_MOUSE )
		{
			// mouse_joint.c:77-128
			float4 d1 = w.jdef1[j]; // target.xy hertz dampingRatio
			Soft ls = make_soft( d1.z, d1.w, h );
			Soft as = make_soft( 0.5f, 0.1f, h );
			fv2 rB = anchorB;
			fv2 cx, cy;
			cx.x = mB + iB * rB.y * rB.y;
			cx.y = -iB * rB.x * rB.y;
			cy.x = cx.y;
			cy.y = mB + iB * rB.x * rB.x;
			fv2 dc = vsub( mk( cb.x, cb.y ), mk( d1.x, d1.y ) );
			w.jprep0[j] = make_float4( anchorA.x, anchorA.y, anchorB.x, anchorB.y );
			w.jprep1[j] = make_float4( dc.x, dc.y, 0.0f, 0.0f );
			w.jprep2[j] = make_float4( ls.biasRate, ls.massScale, ls.impulseScale, 0.0f );
			w.jprep2[w.jointCap + j] = make_float4( as.biasRate, as.massScale, as.impulseScale, 0.0f );
			w.jprep3[j] = inverse22( cx, cy );
			if ( w.enableWarmStarting == 0 )
				w.jimp[j] = make_float4( 0.0f, 0.0f, 0.0f, 0.0f );
			continue;
		}
		if ( type == JT_FILTER )
			continue;
		if ( type == JT_DISTANCE )
		{
			// distance_joint.c:179-205
			float4 d1 = w.jdef1[j]; // length minLength maxLength hertz
			float4 d2 = w.jdef2[j]; // dampingRatio maxMotorForce motorSpeed
			fv2 separation = vadd( vsub( anchorB, anchorA ), deltaCenter );
			fv2 axis = vnormalize( separation );
			float crA = vcross( anchorA, axis );
			float crB = vcross( anchorB, axis );
			float k = mA + mB + iA * crA * crA + iB * crB * crB;
			float axialMass = k > 0.0f ? 1.0f / k : 0.0f;
			Soft ds = make_soft( d1.w, d2.x, h );
			w.jprep0[j] = make_float4( anchorA.x, anchorA.y, anchorB.x, anchorB.y );
			w.jprep1[j] = make_float4( deltaCenter.x, deltaCenter.y, 0.0f, axialMass );
			w.jprep2[j] = make_float4( ds.biasRate, ds.massScale, ds.impulseScale, 0.0f );
			w.jprep2[w.jointCap + j] =
				make_float4( jointSoft.biasRate, jointSoft.massScale, jointSoft.impulseScale, 0.0f );
			if ( w.enableWarmStarting == 0 )
				w.jimp[j] = make_float4( 0.0f, 0.0f, 0.0f, 0.0f );
			continue;
		}
		float deltaAngle = relative_angle( qB, qA );
		float k = iA + iB;
		float axialMass = k > 0.0f ? 1.0f / k : 0.0f;
		float4 d1 = w.jdef1[j];
		Soft spring = make_soft( d1.z, d1.w, h );
		w.jprep0[j] = make_float4( anchorA.x, anchorA.y, anchorB.x, anchorB.y );
		w.jprep1[j] = make_float4( deltaCenter.x, deltaCenter.y, deltaAngle, axialMass );
		w.jprep2[j] = make_float4( spring.biasRate, spring.massScale, spring.impulseScale, 0.0f );
		w.jprep2[w.jointCap + j] = make_float4( jointSoft.biasRate, jointSoft.massScale, jointSoft.impulseScale, 0.0f );
		if ( w.enableWarmStarting == 0 )
		{
			w.jimp[j] = make_float4( 0.0f, 0.0f, 0.0f, 0.0f );
			w.jimp2[j] = make_float2( 0.0f, 0.0f );
		}
	}
}

__global__ void k_joint_count( DWorld w, int* cnt )
{
	int n = w.jointCount;
	for ( int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x )
	{
		int c = w.jcolor[j];
		if ( ( w.jflags[j] & JF_USED ) && c >= 0 && c < F2D_OVERFLOW )
			atomicAdd( cnt + c, 1 );
	}
}

__global__ void k_joint_offsets( int* cnt, int* start )
{
	if ( threadIdx.x != 0 || blockIdx.x != 0 )
		return;
	int s = 0;
	for ( int c = 0; c < F2D_OVERFLOW; ++c )
	{
		start[c] = s;
		s += cnt[c];
		cnt[c] = 0;
	}
	start[F2D_OVERFLOW] = s;
}

__global__ void k_joint_fill( DWorld w, int* cnt, const int* start, int* slots )
{
	int n = w.jointCount;
	for ( int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x )
	{
		int c = w.jcolor[j];
		if ( ( w.jflags[j] & JF_USED ) && c >= 0 && c < F2D_OVERFLOW )
			slots[start[c] + atomicAdd( cnt + c, 1 )] = j;
	}
}

__global__ void k_zero_small( int* p, int n )
{
	if ( threadIdx.x < n )
		p[threadIdx.x] = 0;
}

void launch_prepare_joints( DWorld& w, StepScratch& s, cudaStream_t st, float h, float inv_h, Soft jointSoft )
{
	int* slots = s.tmpB;
	int* start = s.tmpB + w.jointCap;
	int* cnt = start + F2D_COLORS + 4;
	k_zero_small<<<1, 32, 0, st>>>( cnt, F2D_COLORS );
	if ( w.jointCount > 0 )
	{
		k_prepare_joints<<<grid_for( w.jointCount ), 256, 0, st>>>( w, h, inv_h, jointSoft );
		k_joint_count<<<grid_for( w.jointCount ), 256, 0, st>>>( w, cnt );
	}
	k_joint_offsets<<<1, 1, 0, st>>>( cnt, start );
	if ( w.jointCount > 0 )
		k_joint_fill<<<grid_for( w.jointCount ), 256, 0, st>>>( w, cnt, start, slots );
}
