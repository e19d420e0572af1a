// Soft-step solver of the world step, GPU-first.
//
// Stage order is that of b2SolverTask (packages/forge2d/third_party/box2d/
// src/solver.c:929-1160): prepare joints and contacts; per substep integrate
// velocities, warm start (overflow joints, overflow contacts, then graph
// colours 0..10), solve, integrate positions, relax; then restitution and
// impulse storage. All of it runs in one persistent cooperative kernel: the
// colour stages are separated by grid barriers (bounded spins that raise an
// error bit instead of hanging), the serial overflow constraints run on one
// thread between two barriers, and within a colour one thread solves one
// constraint (bodies within a colour are disjoint, so the slot order inside
// a colour does not change any result).
//
// Constraint arithmetic: graph-colour constraints follow the operand order of
// the reference's SIMD lanes (contact_solver.c:1438-2120, separate mul and
// add, SSE2 min/max/blend semantics); overflow constraints follow its scalar
// functions (contact_solver.c:24-510). Built with -fmad=false the results
// are bit-identical to the reference C code.
#include "dscan.cuh"
#include "dsync.cuh"

#include <cooperative_groups.h>
#include "dworld.cuh"
#include "joint.cuh"
#include "kernels.cuh"


struct SolveParams
{
	float h, inv_h, dt, inv_dt;
	Soft contactSoft, staticSoft, jointSoft;
	float minBiasVel; // -contactSpeed (world.c:767)
	float pushout;	  // maxContactPushSpeed (overflow path)
	float restitutionThreshold;
	float maxLinearSpeed, maxAngularSpeed;
	fv2 gravity;
	int subSteps;
	int enableWarmStarting;
};

// ---------------------------------------------------------------------------
// constraint slots: overflow first (overflow-array order), then colours
// ---------------------------------------------------------------------------
// Colour occupancy of the touching contacts: per-block counts in shared
// memory, one global add per colour and block.
__global__ void k_count_colors( DWorld w, int* fill )
{
	__shared__ int cnt[F2D_OVERFLOW];
	if ( threadIdx.x < F2D_OVERFLOW )
		cnt[threadIdx.x] = 0;
	__syncthreads();
	int n = w.sc->contactIdCount;
	for ( int c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x )
	{
		int col = w.ccolor[c];
		if ( col >= 0 && col < F2D_OVERFLOW && ( w.cflags[c] & CF_USED ) )
			atomicAdd( cnt + col, 1 );
	}
	__syncthreads();
	if ( threadIdx.x < F2D_OVERFLOW && cnt[threadIdx.x] > 0 )
		atomicAdd( fill + threadIdx.x, cnt[threadIdx.x] );
}

__global__ void k_zero_ints( int* p, int n )
{
	for ( int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x )
		p[i] = 0;
}

__global__ void k_color_offsets( DWorld w, int* fill )
{
	if ( blockIdx.x != 0 || threadIdx.x != 0 )
		return;
	int start = w.sc->overflowCount;
	for ( int c = 0; c < F2D_OVERFLOW; ++c )
	{
		w.sc->colorStart[c] = start;
		w.sc->colorCount[c] = fill[c];
		start += fill[c];
		fill[c] = 0;
	}
	w.sc->colorStart[F2D_OVERFLOW] = start;
	w.sc->colorCount[F2D_OVERFLOW] = w.sc->overflowCount;
	w.sc->touchingCount = start;
}

// Constraint slots: overflow contacts first (overflow-array order), then
// each colour's contacts in a contiguous range. Inside a colour the slot
// order is arbitrary (no two constraints of a colour share a dynamic body);
// each block reserves its range with one global add per colour.
__global__ void k_fill_slots( DWorld w, int* fill )
{
	__shared__ int cnt[F2D_OVERFLOW], base[F2D_OVERFLOW];
	int n = w.sc->contactIdCount;
	int nov = w.sc->overflowCount;
	for ( int i = blockIdx.x * blockDim.x + threadIdx.x; i < nov; i += gridDim.x * blockDim.x )
		w.slotContact[i] = w.overflowList[i];
	int stride = gridDim.x * blockDim.x;
	for ( int c0 = blockIdx.x * blockDim.x; c0 < n; c0 += stride )
	{
		if ( threadIdx.x < F2D_OVERFLOW )
			cnt[threadIdx.x] = 0;
		__syncthreads();
		int c = c0 + threadIdx.x;
		int col = -1, rank = 0;
		if ( c < n )
		{
			col = w.ccolor[c];
			if ( col >= 0 && col < F2D_OVERFLOW && ( w.cflags[c] & CF_USED ) )
				rank = atomicAdd( cnt + col, 1 );
			else
				col = -1;
		}
		__syncthreads();
		if ( threadIdx.x < F2D_OVERFLOW )
			base[threadIdx.x] = cnt[threadIdx.x] > 0 ? atomicAdd( fill + threadIdx.x, cnt[threadIdx.x] ) : 0;
		__syncthreads();
		if ( col >= 0 )
			w.slotContact[w.sc->colorStart[col] + base[col] + rank] = c;
		__syncthreads();
	}
}

// contact_solver.c:1438-1669 / :24-156 (identical expressions in both)
__global__ void k_prepare_contacts( DWorld w, SolveParams p )
{
	int n = w.sc->touchingCount;
	float warmStartScale = p.enableWarmStarting ? 1.0f : 0.0f;
	for ( int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x )
	{
		int c = w.slotContact[k];
		int2 bd = w.cbody[c];
		int ia = body_type( w.bflags[bd.x] ) == 0 ? -1 : bd.x;
		int ib = body_type( w.bflags[bd.y] ) == 0 ? -1 : bd.y;
		float4 cm = w.cmass[c];
		float mA = cm.x, iA = cm.y, mB = cm.z, iB = cm.w;
		// constraint_graph.c:139-181: a static side carries zero mass
		if ( ia < 0 )
		{
			mA = 0.0f;
			iA = 0.0f;
		}
		if ( ib < 0 )
		{
			mB = 0.0f;
			iB = 0.0f;
		}
		fv2 vA = mk( 0.0f, 0.0f ), vB = mk( 0.0f, 0.0f );
		float wA = 0.0f, wB = 0.0f;
		if ( ia >= 0 )
		{
			float4 v = w.vel[ia];
			vA = mk( v.x, v.y );
			wA = v.z;
		}
		if ( ib >= 0 )
		{
			float4 v = w.vel[ib];
			vB = mk( v.x, v.y );
			wB = v.z;
		}
		float kk = iA + iB;
		float rollingMass = kk > 0.0f ? 1.0f / kk : 0.0f;
		Soft soft = ( ia < 0 || ib < 0 ) ? p.staticSoft : p.contactSoft;
		float4 mn = w.mnorm[c];
		fv2 normal = mk( mn.x, mn.y );
		int pointCount = __float_as_int( mn.w );
		float4 cmat = w.cmat[c];
		w.kIndex[k] = make_int2( ia, ib );
		w.kMass[k] = make_float4( mA, iA, mB, iB );
		w.kNormal[k] = make_float4( normal.x, normal.y, cmat.x, cmat.w );
		w.kMisc[k] = make_float4( cmat.y, cmat.z, rollingMass, warmStartScale * mn.z );
		w.kSoft[k] = make_float4( soft.biasRate, soft.massScale, soft.impulseScale, __int_as_float( pointCount ) );
		fv2 tangent = vright( normal );
		float4 anch[2], pp[2];
		float ni[2], ti[2];
		for ( int j = 0; j < 2; ++j )
		{
			if ( j >= pointCount )
			{
				anch[j] = make_float4( 0.0f, 0.0f, 0.0f, 0.0f );
				pp[j] = make_float4( 0.0f, 0.0f, 0.0f, 0.0f );
				ni[j] = 0.0f;
				ti[j] = 0.0f;
				continue;
			}
			float4 a = w.mpA[2 * c + j];
			float4 b = w.mpB[2 * c + j];
			float4 im = w.mpI[2 * c + j];
			fv2 rA = mk( a.x, a.y ), rB = mk( a.z, a.w );
			anch[j] = a;
			float baseSeparation = b.z - vdot( vsub( rB, rA ), normal );
			ni[j] = warmStartScale * im.x;
			ti[j] = warmStartScale * im.y;
			float rnA = vcross( rA, normal );
			float rnB = vcross( rB, normal );
			float kNormal = mA + mB + iA * rnA * rnA + iB * rnB * rnB;
			float normalMass = kNormal > 0.0f ? 1.0f / kNormal : 0.0f;
			float rtA = vcross( rA, tangent );
			float rtB = vcross( rB, tangent );
			float kTangent = mA + mB + iA * rtA * rtA + iB * rtB * rtB;
			float tangentMass = kTangent > 0.0f ? 1.0f / kTangent : 0.0f;
			fv2 vrA = vadd( vA, vcrossSV( wA, rA ) );
			fv2 vrB = vadd( vB, vcrossSV( wB, rB ) );
			float relVel = vdot( normal, vsub( vrB, vrA ) );
			pp[j] = make_float4( baseSeparation, normalMass, tangentMass, relVel );
			// learned warm start: features of a point that has no cached impulse
			if ( w.learnMode != 0 && ( ( float_to_bits( b.w ) >> 16 ) & 1 ) == 0 )
			{
				int q = atomicAdd( &w.sc->newPointCount, 1 );
				if ( q < w.newPointCap )
				{
					w.newPoint[q] = make_int2( k, j );
					float* f = w.newFeat + 12 * (size_t)q;
					f[0] = normal.x;
					f[1] = normal.y;
					f[2] = relVel;
					f[3] = vdot( tangent, vsub( vrB, vrA ) );
					f[4] = b.z;
					f[5] = vdot( rA, tangent );
					f[6] = vdot( rB, tangent );
					f[7] = vdot( rA, normal );
					f[8] = vdot( rB, normal );
					f[9] = normalMass;
					f[10] = tangentMass;
					f[11] = cmat.x;
				}
			}
		}
		w.kAnch1[k] = anch[0];
		w.kAnch2[k] = anch[1];
		w.kP1[k] = pp[0];
		w.kP2[k] = pp[1];
		w.kImp[k] = make_float4( ni[0], ni[1], ti[0], ti[1] );
		w.kTot[k] = make_float2( 0.0f, 0.0f );
	}
}

// ---------------------------------------------------------------------------
// body state access: static bodies read as the identity state and are never
// written (contact_solver.c:1184-1222)
// ---------------------------------------------------------------------------

__device__ __forceinline__ BState load_state( const DWorld& w, int i )
{
	BState s;
	if ( i < 0 )
	{
		s.vx = s.vy = s.w = 0.0f;
		s.dpx = s.dpy = 0.0f;
		s.dqc = 1.0f;
		s.dqs = 0.0f;
		return s;
	}
	float4 v = __ldcg( w.vel + i );
	float4 d = __ldcg( w.delta + i );
	s.vx = v.x;
	s.vy = v.y;
	s.w = v.z;
	s.dpx = d.x;
	s.dpy = d.y;
	s.dqc = d.z;
	s.dqs = d.w;
	return s;
}

__device__ __forceinline__ void store_vel( const DWorld& w, int i, const BState& s )
{
	if ( i < 0 )
		return;
	__stcg( w.vel + i, make_float4( s.vx, s.vy, s.w, 0.0f ) );
}

// Body state access of the solver stages. GBodies reads and writes the device
// rows through L2 (.cg); CBodies reads and writes the copy of the body rows
// held in the distributed shared memory of a thread-block cluster (body b in
// block b % F2D_CLUSTER of the cluster, slot b / F2D_CLUSTER; see
// k_solve_cluster). Static bodies (index < 0) read as the identity state and
// are never written.
struct GBodies
{
	float4* vel;
	float4* delta;
	__device__ __forceinline__ BState load( int i ) const
	{
		BState s;
		if ( i < 0 )
		{
			s.vx = s.vy = s.w = 0.0f;
			s.dpx = s.dpy = 0.0f;
			s.dqc = 1.0f;
			s.dqs = 0.0f;
			return s;
		}
		float4 v = __ldcg( vel + i );
		float4 d = __ldcg( delta + i );
		s.vx = v.x;
		s.vy = v.y;
		s.w = v.z;
		s.dpx = d.x;
		s.dpy = d.y;
		s.dqc = d.z;
		s.dqs = d.w;
		return s;
	}
	__device__ __forceinline__ void store( int i, const BState& s ) const
	{
		if ( i >= 0 )
			__stcg( vel + i, make_float4( s.vx, s.vy, s.w, 0.0f ) );
	}
};

#define F2D_CLUSTER 16

__device__ __forceinline__ unsigned dsm_map( unsigned localAddr, unsigned rank )
{
	unsigned r;
	asm volatile( "mapa.shared::cluster.u32 %0, %1, %2;" : "=r"( r ) : "r"( localAddr ), "r"( rank ) );
	return r;
}

__device__ __forceinline__ float4 dsm_ld4( unsigned addr )
{
	float4 v;
	asm volatile( "ld.shared::cluster.v4.f32 {%0, %1, %2, %3}, [%4];"
				  : "=f"( v.x ), "=f"( v.y ), "=f"( v.z ), "=f"( v.w )
				  : "r"( addr )
				  : "memory" );
	return v;
}

__device__ __forceinline__ void dsm_st4( unsigned addr, float4 v )
{
	asm volatile( "st.shared::cluster.v4.f32 [%0], {%1, %2, %3, %4};" ::"r"( addr ), "f"( v.x ), "f"( v.y ), "f"( v.z ),
				  "f"( v.w )
				  : "memory" );
}

struct CBodies
{
	unsigned base; // shared::cta address of this block's slots (vel, delta per slot)
	__device__ __forceinline__ unsigned addr( int i ) const
	{
		return dsm_map( base + 32u * (unsigned)( i / F2D_CLUSTER ), (unsigned)( i % F2D_CLUSTER ) );
	}
	__device__ __forceinline__ BState load( int i ) const
	{
		BState s;
		if ( i < 0 )
		{
			s.vx = s.vy = s.w = 0.0f;
			s.dpx = s.dpy = 0.0f;
			s.dqc = 1.0f;
			s.dqs = 0.0f;
			return s;
		}
		unsigned a = addr( i );
		float4 v = dsm_ld4( a );
		float4 d = dsm_ld4( a + 16u );
		s.vx = v.x;
		s.vy = v.y;
		s.w = v.z;
		s.dpx = d.x;
		s.dpy = d.y;
		s.dqc = d.z;
		s.dqs = d.w;
		return s;
	}
	__device__ __forceinline__ void store( int i, const BState& s ) const
	{
		if ( i >= 0 )
			dsm_st4( addr( i ), make_float4( s.vx, s.vy, s.w, 0.0f ) );
	}
};

__device__ __forceinline__ float lmax( float a, float b )
{
	return a > b ? a : b;
}
__device__ __forceinline__ float lmin( float a, float b )
{
	return a < b ? a : b;
}

// A graph-colour constraint held in registers for the whole solver launch:
// its static rows are read once, its impulses accumulate in place and are
// written back once (see k_solve).
struct Lane
{
	int2 idx;
	float4 ms;	 // invMassA invIA invMassB invIB
	float4 nm;	 // normal.xy friction tangentSpeed
	float4 sf;	 // biasRate massScale impulseScale pointCount
	float4 misc; // restitution rollingResistance rollingMass rollingImpulse
	float4 imp;	 // normalImpulse1 normalImpulse2 tangentImpulse1 tangentImpulse2
	float2 tot;	 // totalNormalImpulse1 totalNormalImpulse2
	float4 an[2];
	float4 pt[2];
};

__device__ __forceinline__ void lane_load( const DWorld& w, int k, Lane& L )
{
	L.idx = w.kIndex[k];
	L.ms = w.kMass[k];
	L.nm = w.kNormal[k];
	L.sf = w.kSoft[k];
	L.misc = __ldcg( w.kMisc + k );
	L.imp = __ldcg( w.kImp + k );
	L.tot = __ldcg( w.kTot + k );
	L.an[0] = w.kAnch1[k];
	L.an[1] = w.kAnch2[k];
	L.pt[0] = w.kP1[k];
	L.pt[1] = w.kP2[k];
}

__device__ __forceinline__ void lane_store( const DWorld& w, int k, const Lane& L )
{
	__stcg( w.kImp + k, L.imp );
	__stcg( w.kTot + k, L.tot );
	__stcg( w.kMisc + k, L.misc );
}

// contact_solver.c:1671-1727
template <class BA> __device__ __forceinline__ void lane_warm( const BA& ba, const Lane& L )
{
	BState A = ba.load( L.idx.x ), B = ba.load( L.idx.y );
	const float4 ms = L.ms, nm = L.nm;
	float tx = nm.y;
	float ty = 0.0f - nm.x;
	float nis[2] = { L.imp.x, L.imp.y };
	float tis[2] = { L.imp.z, L.imp.w };
	for ( int j = 0; j < 2; ++j )
	{
		float rAx = L.an[j].x, rAy = L.an[j].y, rBx = L.an[j].z, rBy = L.an[j].w;
		float Px = nis[j] * nm.x + tis[j] * tx;
		float Py = nis[j] * nm.y + tis[j] * ty;
		A.w = A.w - ms.y * ( rAx * Py - rAy * Px );
		A.vx = A.vx - ms.x * Px;
		A.vy = A.vy - ms.x * Py;
		B.w = B.w + ms.w * ( rBx * Py - rBy * Px );
		B.vx = B.vx + ms.z * Px;
		B.vy = B.vy + ms.z * Py;
	}
	A.w = A.w - ms.y * L.misc.w;
	B.w = B.w + ms.w * L.misc.w;
	ba.store( L.idx.x, A );
	ba.store( L.idx.y, B );
}

// contact_solver.c:1729-1967
template <class BA>
__device__ __forceinline__ void lane_solve( const BA& ba, Lane& L, float inv_h, float minBiasVel, bool useBias )
{
	BState A = ba.load( L.idx.x ), B = ba.load( L.idx.y );
	const float4 ms = L.ms, nm = L.nm, sf = L.sf;
	float4 misc = L.misc;
	float biasRate, massScale, impulseScale;
	if ( useBias )
	{
		biasRate = sf.x;
		massScale = sf.y;
		impulseScale = sf.z;
	}
	else
	{
		biasRate = 0.0f;
		massScale = 1.0f;
		impulseScale = 0.0f;
	}
	float totalNormalImpulse = 0.0f;
	float dpx = B.dpx - A.dpx;
	float dpy = B.dpy - A.dpy;
	float nis[2] = { L.imp.x, L.imp.y };
	float tis[2] = { L.imp.z, L.imp.w };
	float tots[2] = { L.tot.x, L.tot.y };
	for ( int j = 0; j < 2; ++j )
	{
		float rAx = L.an[j].x, rAy = L.an[j].y, rBx = L.an[j].z, rBy = L.an[j].w;
		float rsAx = A.dqc * rAx - A.dqs * rAy;
		float rsAy = A.dqs * rAx + A.dqc * rAy;
		float rsBx = B.dqc * rBx - B.dqs * rBy;
		float rsBy = B.dqs * rBx + B.dqc * rBy;
		float dsx = dpx + ( rsBx - rsAx );
		float dsy = dpy + ( rsBy - rsAy );
		float s = ( nm.x * dsx + nm.y * dsy ) + L.pt[j].x;
		bool mask = s > 0.0f;
		float specBias = s * inv_h;
		float softBias = lmax( biasRate * s, minBiasVel );
		float bias = mask ? specBias : softBias;
		float pointMassScale = mask ? 1.0f : massScale;
		float pointImpulseScale = mask ? 0.0f : impulseScale;
		float dvx = ( B.vx - B.w * rBy ) - ( A.vx - A.w * rAy );
		float dvy = ( B.vy + B.w * rBx ) - ( A.vy + A.w * rAx );
		float vn = dvx * nm.x + dvy * nm.y;
		float negImpulse = L.pt[j].y * ( pointMassScale * ( vn + bias ) ) + pointImpulseScale * nis[j];
		float newImpulse = lmax( nis[j] - negImpulse, 0.0f );
		float impulse = newImpulse - nis[j];
		nis[j] = newImpulse;
		tots[j] = tots[j] + newImpulse;
		totalNormalImpulse = totalNormalImpulse + newImpulse;
		float Px = impulse * nm.x;
		float Py = impulse * nm.y;
		A.vx = A.vx - ms.x * Px;
		A.vy = A.vy - ms.x * Py;
		A.w = A.w - ms.y * ( rAx * Py - rAy * Px );
		B.vx = B.vx + ms.z * Px;
		B.vy = B.vy + ms.z * Py;
		B.w = B.w + ms.w * ( rBx * Py - rBy * Px );
	}
	float tx = nm.y;
	float ty = 0.0f - nm.x;
	for ( int j = 0; j < 2; ++j )
	{
		float rAx = L.an[j].x, rAy = L.an[j].y, rBx = L.an[j].z, rBy = L.an[j].w;
		float dvx = ( B.vx - B.w * rBy ) - ( A.vx - A.w * rAy );
		float dvy = ( B.vy + B.w * rBx ) - ( A.vy + A.w * rAx );
		float vt = dvx * tx + dvy * ty;
		vt = vt - nm.w;
		float negImpulse = L.pt[j].z * vt;
		float maxFriction = nm.z * nis[j];
		float newImpulse = tis[j] - negImpulse;
		newImpulse = lmax( 0.0f - maxFriction, lmin( newImpulse, maxFriction ) );
		float impulse = newImpulse - tis[j];
		tis[j] = newImpulse;
		float Px = impulse * tx;
		float Py = impulse * ty;
		A.vx = A.vx - ms.x * Px;
		A.vy = A.vy - ms.x * Py;
		A.w = A.w - ms.y * ( rAx * Py - rAy * Px );
		B.vx = B.vx + ms.z * Px;
		B.vy = B.vy + ms.z * Py;
		B.w = B.w + ms.w * ( rBx * Py - rBy * Px );
	}
	{
		float deltaLambda = misc.z * ( A.w - B.w );
		float lambda = misc.w;
		float maxLambda = misc.y * totalNormalImpulse;
		float nb = -maxLambda;
		float r = lmax( nb, lmin( lambda + deltaLambda, maxLambda ) );
		misc.w = r;
		deltaLambda = r - lambda;
		A.w = A.w - ms.y * deltaLambda;
		B.w = B.w + ms.w * deltaLambda;
	}
	L.imp = make_float4( nis[0], nis[1], tis[0], tis[1] );
	L.tot = make_float2( tots[0], tots[1] );
	L.misc = misc;
	ba.store( L.idx.x, A );
	ba.store( L.idx.y, B );
}

// contact_solver.c:1969-2076 (lanes with restitution 0 are unchanged)
template <class BA> __device__ __forceinline__ void lane_restitution( const BA& ba, Lane& L, float threshold )
{
	float restitution = L.misc.x;
	if ( restitution == 0.0f )
		return;
	BState A = ba.load( L.idx.x ), B = ba.load( L.idx.y );
	const float4 ms = L.ms, nm = L.nm;
	float nis[2] = { L.imp.x, L.imp.y };
	float tots[2] = { L.tot.x, L.tot.y };
	for ( int j = 0; j < 2; ++j )
	{
		bool mask1 = ( L.pt[j].w + threshold ) > 0.0f;
		bool mask2 = tots[j] == 0.0f;
		float mass = ( mask1 || mask2 ) ? 0.0f : L.pt[j].y;
		float rAx = L.an[j].x, rAy = L.an[j].y, rBx = L.an[j].z, rBy = L.an[j].w;
		float dvx = ( B.vx - B.w * rBy ) - ( A.vx - A.w * rAy );
		float dvy = ( B.vy + B.w * rBx ) - ( A.vy + A.w * rAx );
		float vn = dvx * nm.x + dvy * nm.y;
		float negImpulse = mass * ( vn + restitution * L.pt[j].w );
		float newImpulse = lmax( nis[j] - negImpulse, 0.0f );
		float impulse = newImpulse - nis[j];
		nis[j] = newImpulse;
		float Px = impulse * nm.x;
		float Py = impulse * nm.y;
		A.vx = A.vx - ms.x * Px;
		A.vy = A.vy - ms.x * Py;
		A.w = A.w - ms.y * ( rAx * Py - rAy * Px );
		B.vx = B.vx + ms.z * Px;
		B.vy = B.vy + ms.z * Py;
		B.w = B.w + ms.w * ( rBx * Py - rBy * Px );
	}
	L.imp.x = nis[0];
	L.imp.y = nis[1];
	ba.store( L.idx.x, A );
	ba.store( L.idx.y, B );
}

// contact_solver.c:160-225
template <class BA> static __device__ void warm_overflow( const DWorld& w, const BA& ba, int k )
{
	int2 idx = w.kIndex[k];
	BState A = ba.load( idx.x ), B = ba.load( idx.y );
	float4 ms = w.kMass[k];
	float4 nm = w.kNormal[k];
	float4 imp = __ldcg( w.kImp + k );
	float4 misc = __ldcg( w.kMisc + k );
	int count = __float_as_int( w.kSoft[k].w );
	fv2 normal = mk( nm.x, nm.y );
	fv2 tangent = vright( normal );
	fv2 vA = mk( A.vx, A.vy ), vB = mk( B.vx, B.vy );
	float wA = A.w, wB = B.w;
	float4 an[2] = { w.kAnch1[k], w.kAnch2[k] };
	float nis[2] = { imp.x, imp.y };
	float tis[2] = { imp.z, imp.w };
	for ( int j = 0; j < count; ++j )
	{
		fv2 rA = mk( an[j].x, an[j].y ), rB = mk( an[j].z, an[j].w );
		fv2 P = vadd( vscale( nis[j], normal ), vscale( tis[j], tangent ) );
		wA -= ms.y * vcross( rA, P );
		vA = vmuladd( vA, -ms.x, P );
		wB += ms.w * vcross( rB, P );
		vB = vmuladd( vB, ms.z, P );
	}
	wA -= ms.y * misc.w;
	wB += ms.w * misc.w;
	A.vx = vA.x;
	A.vy = vA.y;
	A.w = wA;
	B.vx = vB.x;
	B.vy = vB.y;
	B.w = wB;
	ba.store( idx.x, A );
	ba.store( idx.y, B );
}

// contact_solver.c:227-380
template <class BA>
static __device__ void solve_overflow( const DWorld& w, const BA& ba, int k, float inv_h, float pushout, bool useBias )
{
	int2 idx = w.kIndex[k];
	BState A = ba.load( idx.x ), B = ba.load( idx.y );
	float4 ms = w.kMass[k];
	float mA = ms.x, iA = ms.y, mB = ms.z, iB = ms.w;
	float4 nm = w.kNormal[k];
	float4 sf = w.kSoft[k];
	float4 misc = __ldcg( w.kMisc + k );
	float4 imp = __ldcg( w.kImp + k );
	float2 tot = __ldcg( w.kTot + k );
	int count = __float_as_int( sf.w );
	fv2 vA = mk( A.vx, A.vy ), vB = mk( B.vx, B.vy );
	float wA = A.w, wB = B.w;
	frot dqA, dqB;
	dqA.c = A.dqc;
	dqA.s = A.dqs;
	dqB.c = B.dqc;
	dqB.s = B.dqs;
	fv2 dp = vsub( mk( B.dpx, B.dpy ), mk( A.dpx, A.dpy ) );
	fv2 normal = mk( nm.x, nm.y );
	fv2 tangent = vright( normal );
	float friction = nm.z;
	float totalNormalImpulse = 0.0f;
	float4 an[2] = { w.kAnch1[k], w.kAnch2[k] };
	float4 pt[2] = { w.kP1[k], w.kP2[k] };
	float nis[2] = { imp.x, imp.y };
	float tis[2] = { imp.z, imp.w };
	float tots[2] = { tot.x, tot.y };
	for ( int j = 0; j < count; ++j )
	{
		fv2 rA = mk( an[j].x, an[j].y ), rB = mk( an[j].z, an[j].w );
		fv2 ds = vadd( dp, vsub( rrot( dqB, rB ), rrot( dqA, rA ) ) );
		float s = pt[j].x + vdot( ds, normal );
		float velocityBias = 0.0f;
		float massScale = 1.0f;
		float impulseScale = 0.0f;
		if ( s > 0.0f )
			velocityBias = s * inv_h;
		else if ( useBias )
		{
			velocityBias = fmax_s( sf.x * s, -pushout );
			massScale = sf.y;
			impulseScale = sf.z;
		}
		fv2 vrA = vadd( vA, vcrossSV( wA, rA ) );
		fv2 vrB = vadd( vB, vcrossSV( wB, rB ) );
		float vn = vdot( vsub( vrB, vrA ), normal );
		float impulse = -pt[j].y * massScale * ( vn + velocityBias ) - impulseScale * nis[j];
		float newImpulse = fmax_s( nis[j] + impulse, 0.0f );
		impulse = newImpulse - nis[j];
		nis[j] = newImpulse;
		tots[j] += newImpulse;
		totalNormalImpulse += newImpulse;
		fv2 P = vscale( impulse, normal );
		vA = vmulsub( vA, mA, P );
		wA -= iA * vcross( rA, P );
		vB = vmuladd( vB, mB, P );
		wB += iB * vcross( rB, P );
	}
	for ( int j = 0; j < count; ++j )
	{
		fv2 rA = mk( an[j].x, an[j].y ), rB = mk( an[j].z, an[j].w );
		fv2 vrB = vadd( vB, vcrossSV( wB, rB ) );
		fv2 vrA = vadd( vA, vcrossSV( wA, rA ) );
		float vt = vdot( vsub( vrB, vrA ), tangent ) - nm.w;
		float impulse = pt[j].z * ( -vt );
		float maxFriction = friction * nis[j];
		float newImpulse = fclamp_s( tis[j] + impulse, -maxFriction, maxFriction );
		impulse = newImpulse - tis[j];
		tis[j] = newImpulse;
		fv2 P = vscale( impulse, tangent );
		vA = vmulsub( vA, mA, P );
		wA -= iA * vcross( rA, P );
		vB = vmuladd( vB, mB, P );
		wB += iB * vcross( rB, P );
	}
	{
		float deltaLambda = -misc.z * ( wB - wA );
		float lambda = misc.w;
		float maxLambda = misc.y * totalNormalImpulse;
		misc.w = fclamp_s( lambda + deltaLambda, -maxLambda, maxLambda );
		deltaLambda = misc.w - lambda;
		wA -= iA * deltaLambda;
		wB += iB * deltaLambda;
	}
	__stcg( w.kImp + k, make_float4( nis[0], nis[1], tis[0], tis[1] ) );
	__stcg( w.kTot + k, make_float2( tots[0], tots[1] ) );
	__stcg( w.kMisc + k, misc );
	A.vx = vA.x;
	A.vy = vA.y;
	A.w = wA;
	B.vx = vB.x;
	B.vy = vB.y;
	B.w = wB;
	ba.store( idx.x, A );
	ba.store( idx.y, B );
}

// contact_solver.c:382-478
template <class BA> static __device__ void restitution_overflow( const DWorld& w, const BA& ba, int k, float threshold )
{
	float4 misc = __ldcg( w.kMisc + k );
	float restitution = misc.x;
	if ( restitution == 0.0f )
		return;
	int2 idx = w.kIndex[k];
	BState A = ba.load( idx.x ), B = ba.load( idx.y );
	float4 ms = w.kMass[k];
	float mA = ms.x, iA = ms.y, mB = ms.z, iB = ms.w;
	float4 nm = w.kNormal[k];
	int count = __float_as_int( w.kSoft[k].w );
	float4 imp = __ldcg( w.kImp + k );
	float2 tot = __ldcg( w.kTot + k );
	fv2 vA = mk( A.vx, A.vy ), vB = mk( B.vx, B.vy );
	float wA = A.w, wB = B.w;
	fv2 normal = mk( nm.x, nm.y );
	float4 an[2] = { w.kAnch1[k], w.kAnch2[k] };
	float4 pt[2] = { w.kP1[k], w.kP2[k] };
	float nis[2] = { imp.x, imp.y };
	float tots[2] = { tot.x, tot.y };
	for ( int j = 0; j < count; ++j )
	{
		if ( pt[j].w > -threshold || tots[j] == 0.0f )
			continue;
		fv2 rA = mk( an[j].x, an[j].y ), rB = mk( an[j].z, an[j].w );
		fv2 vrB = vadd( vB, vcrossSV( wB, rB ) );
		fv2 vrA = vadd( vA, vcrossSV( wA, rA ) );
		float vn = vdot( vsub( vrB, vrA ), normal );
		float impulse = -pt[j].y * ( vn + restitution * pt[j].w );
		float newImpulse = fmax_s( nis[j] + impulse, 0.0f );
		impulse = newImpulse - nis[j];
		nis[j] = newImpulse;
		tots[j] += impulse;
		fv2 P = vscale( impulse, normal );
		vA = vmulsub( vA, mA, P );
		wA -= iA * vcross( rA, P );
		vB = vmuladd( vB, mB, P );
		wB += iB * vcross( rB, P );
	}
	__stcg( w.kImp + k, make_float4( nis[0], nis[1], imp.z, imp.w ) );
	__stcg( w.kTot + k, make_float2( tots[0], tots[1] ) );
	A.vx = vA.x;
	A.vy = vA.y;
	A.w = wA;
	B.vx = vB.x;
	B.vy = vB.y;
	B.w = wB;
	ba.store( idx.x, A );
	ba.store( idx.y, B );
}

// ---------------------------------------------------------------------------
// Overflow levels. The reference solves the overflow joints and then the
// overflow contacts one after another on its main thread (solver.c:1008-1009,
// 1027-1028, 1055-1056, 1077). Here those constraints are split into levels:
// constraint e (joints first, then contacts, each in overflow-array order)
// joins level r when every earlier overflow constraint that shares a
// non-static body with it sits in a level below r (as-soon-as-possible
// scheduling of each body's constraint order). Constraints of one level touch
// disjoint bodies and every body meets its constraints in the serial order,
// so one block solving the levels one after another, with a block barrier
// between levels, produces the serial sweep's values bit for bit.
#define OVF_MAX_LEVELS 64	 // rounds of level assignment; the rest go serial
#define OVF_SMEM_ITEMS 3072 // level-ordered list kept in shared memory

struct OvfPlan
{
	const int* order; // constraints in level order
	int levels;		  // parallel levels
	int n;			  // overflow joints + contacts
	int nj;			  // overflow joints
};

static __device__ __forceinline__ int2 ovf_bodies( const DWorld& w, int e, int nj )
{
	return e < nj ? w.jindex[w.overflowJoints[e]] : w.kIndex[e - nj];
}

// All threads of one block. Writes the level-ordered list into order (n
// entries) and the level starts into levelStart (OVF_MAX_LEVELS + 1 entries,
// shared memory). Constraints left after OVF_MAX_LEVELS rounds follow in
// ascending order as one serial tail.
static __device__ OvfPlan ovf_schedule( const DWorld& w, int* order, int* levelStart )
{
	__shared__ int sPos;
	OvfPlan plan;
	plan.nj = w.sc->overflowJointCount;
	plan.n = plan.nj + w.sc->overflowCount;
	plan.order = order;
	const int n = plan.n, nj = plan.nj;
	int* level = w.ovfLevel;
	int* owner = w.ovfOwner;
	for ( int e = threadIdx.x; e < n; e += blockDim.x )
		__stcg( level + e, -1 );
	if ( threadIdx.x == 0 )
	{
		sPos = 0;
		levelStart[0] = 0;
	}
	__syncthreads();
	int r = 0;
	while ( r < OVF_MAX_LEVELS && sPos < n )
	{
		for ( int e = threadIdx.x; e < n; e += blockDim.x )
			if ( __ldcg( level + e ) < 0 )
			{
				int2 b = ovf_bodies( w, e, nj );
				if ( b.x >= 0 )
					__stcg( owner + b.x, 0x7fffffff );
				if ( b.y >= 0 )
					__stcg( owner + b.y, 0x7fffffff );
			}
		__syncthreads();
		for ( int e = threadIdx.x; e < n; e += blockDim.x )
			if ( __ldcg( level + e ) < 0 )
			{
				int2 b = ovf_bodies( w, e, nj );
				if ( b.x >= 0 )
					atomicMin( owner + b.x, e );
				if ( b.y >= 0 )
					atomicMin( owner + b.y, e );
			}
		__syncthreads();
		for ( int e = threadIdx.x; e < n; e += blockDim.x )
			if ( __ldcg( level + e ) < 0 )
			{
				int2 b = ovf_bodies( w, e, nj );
				bool first = ( b.x < 0 || __ldcg( owner + b.x ) == e ) && ( b.y < 0 || __ldcg( owner + b.y ) == e );
				if ( first )
				{
					__stcg( level + e, r );
					order[atomicAdd( &sPos, 1 )] = e;
				}
			}
		__syncthreads();
		r += 1;
		if ( threadIdx.x == 0 )
			levelStart[r] = sPos;
		__syncthreads();
	}
	plan.levels = r;
	if ( threadIdx.x == 0 && sPos < n )
	{
		int pos = sPos;
		for ( int e = 0; e < n; ++e )
			if ( __ldcg( level + e ) < 0 )
				order[pos++] = e;
	}
	__syncthreads();
	return plan;
}

// kind 0 warm start, 1 solve, 2 relax, 3 restitution (contacts only)
template <class BA>
static __device__ __forceinline__ void ovf_item( const DWorld& w, const BA& ba, int e, int nj, int kind,
												  const SolveParams& p )
{
	if ( e < nj )
	{
		int j = w.overflowJoints[e];
		if ( kind == 0 )
			joint_warm_start( w, ba, j );
		else if ( kind < 3 )
			joint_solve( w, ba, j, p.h, p.inv_h, kind == 1 );
		return;
	}
	int k = e - nj;
	if ( kind == 0 )
		warm_overflow( w, ba, k );
	else if ( kind < 3 )
		solve_overflow( w, ba, k, p.inv_h, p.pushout, kind == 1 );
	else
		restitution_overflow( w, ba, k, p.restitutionThreshold );
}

// All threads of the scheduling block: the overflow constraints level by
// level, then the serial tail on thread 0.
template <class BA>
static __device__ void ovf_stage( const DWorld& w, const BA& ba, const OvfPlan& plan, const int* levelStart, int kind,
								  const SolveParams& p )
{
	for ( int l = 0; l < plan.levels; ++l )
	{
		int end = levelStart[l + 1];
		for ( int i = levelStart[l] + threadIdx.x; i < end; i += blockDim.x )
			ovf_item( w, ba, plan.order[i], plan.nj, kind, p );
		__syncthreads();
	}
	if ( threadIdx.x == 0 )
		for ( int i = levelStart[plan.levels]; i < plan.n; ++i )
			ovf_item( w, ba, plan.order[i], plan.nj, kind, p );
	__syncthreads();
}

__device__ __forceinline__ void integrate_velocity( const DWorld& w, int b, const SolveParams& p )
{
	float4 v4 = w.vel[b];
	float4 m = w.massv[b];
	float4 dmp = w.damp[b];
	float4 f = w.force[b];
	float h = p.h;
	float maxLinearSpeedSq = p.maxLinearSpeed * p.maxLinearSpeed;
	float maxAngularSpeedSq = p.maxAngularSpeed * p.maxAngularSpeed;
	fv2 v = mk( v4.x, v4.y );
	float wv = v4.z;
	float linearDamping = 1.0f / ( 1.0f + h * dmp.x );
	float angularDamping = 1.0f / ( 1.0f + h * dmp.y );
	float gravityScale = m.x > 0.0f ? dmp.z : 0.0f;
	fv2 g = p.gravity;
	if ( w.subCount > 0 )
	{
		float2 gb = w.bodyGravity[b];
		g = mk( gb.x, gb.y );
	}
	fv2 lvd = vadd( vscale( h * m.x, mk( f.x, f.y ) ), vscale( h * gravityScale, g ) );
	float avd = h * m.y * f.z;
	v = vmuladd( lvd, linearDamping, v );
	wv = avd + angularDamping * wv;
	int flags = w.bflags[b];
	bool capped = false;
	if ( vdot( v, v ) > maxLinearSpeedSq )
	{
		float ratio = p.maxLinearSpeed / vlen( v );
		v = vscale( ratio, v );
		capped = true;
	}
	if ( wv * wv > maxAngularSpeedSq && ( flags & BF_FAST_ROT ) == 0 )
	{
		float ratio = p.maxAngularSpeed / fabs_s( wv );
		wv *= ratio;
		capped = true;
	}
	if ( capped )
		w.bflags[b] = flags | BF_SPEED_CAPPED;
	w.vel[b] = make_float4( v.x, v.y, wv, 0.0f );
}

__device__ __forceinline__ bool body_awake( int f )
{
	return ( f & ( BF_USED | BF_ENABLED | BF_ASLEEP ) ) == ( BF_USED | BF_ENABLED ) && body_type( f ) != 0;
}

template <class BA> __device__ __forceinline__ void lane_op( const BA& ba, Lane& L, int kind, const SolveParams& p )
{
	if ( kind == 0 )
		lane_warm( ba, L );
	else if ( kind == 1 )
		lane_solve( ba, L, p.inv_h, p.minBiasVel, true );
	else if ( kind == 2 )
		lane_solve( ba, L, p.inv_h, p.minBiasVel, false );
	else
		lane_restitution( ba, L, p.restitutionThreshold );
}

template <class BA>
__device__ __forceinline__ void joint_colour_stage( const DWorld& w, const BA& ba, int c, int kind, const SolveParams& p,
													int gtid, int gstride, const int* jointSlots, const int* sJStart )
{
	int start = sJStart[c];
	int count = sJStart[c + 1] - start;
	for ( int k = gtid; k < count; k += gstride )
	{
		int j = jointSlots[start + k];
		if ( kind == 0 )
			joint_warm_start( w, ba, j );
		else if ( kind == 1 )
			joint_solve( w, ba, j, p.h, p.inv_h, true );
		else if ( kind == 2 )
			joint_solve( w, ba, j, p.h, p.inv_h, false );
	}
}

// Manifold write-back of one constraint (contact_solver.c:480-509 overflow,
// :2078-2120 graph lanes; graph lanes store both points, zeros for a
// one-point manifold).
__device__ __forceinline__ void store_manifold( const DWorld& w, int k, float4 imp, float2 tot, float rolling,
												float rv1, float rv2, int count, bool lane )
{
	int c = w.slotContact[k];
	w.mpI[2 * c + 0] = make_float4( imp.x, imp.z, tot.x, rv1 );
	if ( lane || count > 1 )
		w.mpI[2 * c + 1] = make_float4( imp.y, imp.w, tot.y, rv2 );
	float4 mn = w.mnorm[c];
	mn.z = rolling;
	w.mnorm[c] = mn;
}

__device__ __forceinline__ void store_manifold_global( const DWorld& w, int k, bool lane )
{
	float4 imp = __ldcg( w.kImp + k );
	float2 tot = __ldcg( w.kTot + k );
	float4 misc = __ldcg( w.kMisc + k );
	store_manifold( w, k, imp, tot, misc.w, w.kP1[k].w, w.kP2[k].w, __float_as_int( w.kSoft[k].w ), lane );
}

// Colour-c constraint slots beyond the register-resident first stride of
// slots: consecutive threads take consecutive slots (coalesced row loads);
// their impulses go through the constraint rows between stages.
template <class BA>
__device__ __forceinline__ void colour_lanes_extra( const DWorld& w, const BA& ba, int c, const int* sStart,
													const int* sCount, int novf, int tid, int stride, int kind,
													const SolveParams& p )
{
	int lo = max( sStart[c], novf + stride ), hi = sStart[c] + sCount[c];
	for ( int k = lo + tid; k < hi; k += stride )
	{
		Lane L;
		if ( kind == 0 )
		{
			// warm start reads no softness or point rows and changes no impulse
			L.idx = w.kIndex[k];
			L.ms = w.kMass[k];
			L.nm = w.kNormal[k];
			L.misc = __ldcg( w.kMisc + k );
			L.imp = __ldcg( w.kImp + k );
			L.an[0] = w.kAnch1[k];
			L.an[1] = w.kAnch2[k];
			lane_warm( ba, L );
			continue;
		}
		lane_load( w, k, L );
		lane_op( ba, L, kind, p );
		if ( kind == 3 )
			__stcg( w.kImp + k, L.imp );
		else
			lane_store( w, k, L );
	}
}

// Tail colours: the highest active colours, without joints, holding at most
// TAIL_MAX constraints together. Block 0 runs them one after another with
// block barriers in between; the grid then needs one barrier for all of
// them instead of one per colour. A constraint's colour and its colour's
// place in the order are unchanged, so results are too.
#define TAIL_MAX 1024

__device__ __forceinline__ int tail_first_colour( const int* sCount, const int* sJStart, unsigned activeMask )
{
	int first = F2D_OVERFLOW, colours = 0, total = 0;
	for ( int c = F2D_OVERFLOW - 1; c >= 0; --c )
	{
		if ( ( activeMask & ( 1u << c ) ) == 0 )
			continue;
		if ( sJStart[c + 1] > sJStart[c] || total + sCount[c] > TAIL_MAX )
			break;
		total += sCount[c];
		first = c;
		colours += 1;
	}
	return colours >= 2 ? first : F2D_OVERFLOW;
}

template <class BA>
__device__ void tail_stage( const DWorld& w, const BA& ba, const int* sStart, const int* sCount, int first,
							unsigned activeMask, int kind, const SolveParams& p )
{
	for ( int c = first; c < F2D_OVERFLOW; ++c )
	{
		if ( ( activeMask & ( 1u << c ) ) == 0 )
			continue;
		for ( int k = sStart[c] + threadIdx.x; k < sStart[c] + sCount[c]; k += blockDim.x )
		{
			Lane L;
			if ( kind == 0 )
			{
				L.idx = w.kIndex[k];
				L.ms = w.kMass[k];
				L.nm = w.kNormal[k];
				L.misc = __ldcg( w.kMisc + k );
				L.imp = __ldcg( w.kImp + k );
				L.an[0] = w.kAnch1[k];
				L.an[1] = w.kAnch2[k];
				lane_warm( ba, L );
				continue;
			}
			lane_load( w, k, L );
			lane_op( ba, L, kind, p );
			if ( kind == 3 )
				__stcg( w.kImp + k, L.imp );
			else
				lane_store( w, k, L );
		}
		__syncthreads();
	}
}

// The persistent solver. Graph-colour constraint slots (after the overflow
// slots) are dealt to threads round-robin over the blocks: thread t of block
// b owns colour slot r = t * gridDim.x + b (and r + gridDim.x * blockDim.x,
// ... when the graph holds more constraints than the grid has threads). The
// first owned constraint lives in registers for the whole launch; a colour
// stage then costs one load and one store of each of its two bodies.
template <int THREADS>
__global__ void __launch_bounds__( THREADS ) k_solve( DWorld w, SolveParams p, const int* jointSlots,
													  const int* jointStart )
{
	__shared__ int sStart[F2D_COLORS], sCount[F2D_COLORS], sJStart[F2D_OVERFLOW + 1];
	if ( threadIdx.x < F2D_COLORS )
	{
		sStart[threadIdx.x] = w.sc->colorStart[threadIdx.x];
		sCount[threadIdx.x] = w.sc->colorCount[threadIdx.x];
	}
	if ( threadIdx.x <= F2D_OVERFLOW )
		sJStart[threadIdx.x] = jointStart[threadIdx.x];
	__syncthreads();

	int gtid = blockIdx.x * blockDim.x + threadIdx.x;
	int gstride = gridDim.x * blockDim.x;
	unsigned epoch = 0;
	const GBodies gb = { w.vel, w.delta };
	int nb = w.bodyCount;
	int novf = w.sc->overflowCount;
	int novfJ = w.sc->overflowJointCount;
	int nColour = w.sc->touchingCount - novf;
	bool serialStage = novf > 0 || novfJ > 0;
	unsigned activeMask = 0;
	for ( int c = 0; c < F2D_OVERFLOW; ++c )
		if ( sCount[c] > 0 || sJStart[c + 1] > sJStart[c] )
			activeMask |= 1u << c;
	// block 0 solves the overflow constraints, level by level
	__shared__ int sLevelStart[OVF_MAX_LEVELS + 1];
	__shared__ int sOrder[OVF_SMEM_ITEMS];
	OvfPlan plan = {};
	if ( serialStage && blockIdx.x == 0 )
		plan = ovf_schedule( w, novf + novfJ <= OVF_SMEM_ITEMS ? sOrder : w.ovfOrder, sLevelStart );

	// tail colours run in block 0; their constraints stay in global memory
	const int tailFirst = tail_first_colour( sCount, sJStart, activeMask );
	const int tailSlot = tailFirst < F2D_OVERFLOW ? sStart[tailFirst] : novf + nColour;

	const int r0 = threadIdx.x * gridDim.x + blockIdx.x;
	Lane L0;
	int col0 = -1;
	if ( r0 < nColour && novf + r0 < tailSlot )
	{
		int k0 = novf + r0;
		lane_load( w, k0, L0 );
		for ( int c = 0; c < F2D_OVERFLOW; ++c )
			if ( k0 >= sStart[c] && k0 < sStart[c] + sCount[c] )
				col0 = c;
	}

	for ( int sub = 0; sub < p.subSteps; ++sub )
	{
		for ( int b = gtid; b < nb; b += gstride )
			if ( body_awake( w.bflags[b] ) )
				integrate_velocity( w, b, p );
		if ( !grid_barrier( &w.sc->barrierCount, &w.sc->error, epoch ) )
			return;
		for ( int kind = 0; kind < 3; ++kind )
		{
			if ( kind == 2 )
			{
				// integrate positions (solver.c:182-200)
				for ( int b = gtid; b < nb; b += gstride )
				{
					if ( !body_awake( w.bflags[b] ) )
						continue;
					float4 v = __ldcg( w.vel + b );
					float4 d = __ldcg( w.delta + b );
					frot dq;
					dq.c = d.z;
					dq.s = d.w;
					dq = rintegrate( dq, p.h * v.z );
					fv2 dp = vmuladd( mk( d.x, d.y ), p.h, mk( v.x, v.y ) );
					__stcg( w.delta + b, make_float4( dp.x, dp.y, dq.c, dq.s ) );
				}
				if ( !grid_barrier( &w.sc->barrierCount, &w.sc->error, epoch ) )
					return;
			}
			if ( serialStage )
			{
				if ( blockIdx.x == 0 )
					ovf_stage( w, gb, plan, sLevelStart, kind, p );
				if ( !grid_barrier( &w.sc->barrierCount, &w.sc->error, epoch ) )
					return;
			}
			for ( int c = 0; c < tailFirst; ++c )
			{
				if ( ( activeMask & ( 1u << c ) ) == 0 )
					continue;
				joint_colour_stage( w, gb, c, kind, p, gtid, gstride, jointSlots, sJStart );
				if ( col0 == c )
					lane_op( gb, L0, kind, p );
				colour_lanes_extra( w, gb, c, sStart, sCount, novf, gtid, gstride, kind, p );
				if ( !grid_barrier( &w.sc->barrierCount, &w.sc->error, epoch ) )
					return;
			}
			if ( tailFirst < F2D_OVERFLOW )
			{
				if ( blockIdx.x == 0 )
					tail_stage( w, gb, sStart, sCount, tailFirst, activeMask, kind, p );
				if ( !grid_barrier( &w.sc->barrierCount, &w.sc->error, epoch ) )
					return;
			}
		}
	}
	// restitution: overflow then colours (solver.c:1103-1117)
	if ( novf > 0 )
	{
		if ( blockIdx.x == 0 )
			ovf_stage( w, gb, plan, sLevelStart, 3, p );
		if ( !grid_barrier( &w.sc->barrierCount, &w.sc->error, epoch ) )
			return;
	}
	for ( int c = 0; c < tailFirst; ++c )
	{
		if ( sCount[c] == 0 )
			continue;
		if ( col0 == c )
			lane_op( gb, L0, 3, p );
		colour_lanes_extra( w, gb, c, sStart, sCount, novf, gtid, gstride, 3, p );
		if ( !grid_barrier( &w.sc->barrierCount, &w.sc->error, epoch ) )
			return;
	}
	if ( tailFirst < F2D_OVERFLOW )
	{
		if ( blockIdx.x == 0 )
			tail_stage( w, gb, sStart, sCount, tailFirst, activeMask, 3, p );
		if ( !grid_barrier( &w.sc->barrierCount, &w.sc->error, epoch ) )
			return;
	}
	// store impulses into the manifolds
	for ( int k = gtid; k < novf; k += gstride )
		store_manifold_global( w, k, false );
	if ( col0 >= 0 )
		store_manifold( w, novf + r0, L0.imp, L0.tot, L0.misc.w, L0.pt[0].w, L0.pt[1].w,
						__float_as_int( L0.sf.w ), true );
	for ( int k = novf + gstride + gtid; k < novf + nColour; k += gstride )
		store_manifold_global( w, k, true );
	// tail constraints below the extras' range had no register lane
	for ( int k = tailSlot + gtid; k < min( novf + gstride, novf + nColour ); k += gstride )
		store_manifold_global( w, k, true );
	if ( blockIdx.x == 0 && threadIdx.x == 0 )
		w.sc->solveBarriers = (int)epoch; // grid barriers this launch passed
}

// A launch of nothing but grid barriers on the solver's grid: the per-barrier
// latency that bounds the stages of k_solve from below.
__global__ void __launch_bounds__( 512 ) k_barrier_probe( unsigned* counter, int* err, int n )
{
	unsigned epoch = 0;
	for ( int i = 0; i < n; ++i )
		if ( !grid_barrier( counter, err, epoch ) )
			return;
}

float solver_barrier_probe( StepScratch& s, cudaStream_t st, unsigned* counter, int* err, int n )
{
	cudaEvent_t a, b;
	cudaEventCreate( &a );
	cudaEventCreate( &b );
	cudaMemsetAsync( counter, 0, sizeof( unsigned ), st );
	void* args[] = { &counter, &err, &n };
	cudaEventRecord( a, st );
	cudaLaunchCooperativeKernel( (void*)k_barrier_probe, dim3( s.solverBlocks ), dim3( 512 ), args, 0, st );
	cudaEventRecord( b, st );
	cudaEventSynchronize( b );
	float ms = 0.0f;
	cudaEventElapsedTime( &ms, a, b );
	cudaEventDestroy( a );
	cudaEventDestroy( b );
	return n > 0 ? 1000.0f * ms / (float)n : 0.0f;
}

// ---------------------------------------------------------------------------
// Cluster solver: the same stages on one thread-block cluster of F2D_CLUSTER
// blocks, for worlds whose body rows fit the cluster's shared memory. The
// body velocities and substep deltas live in distributed shared memory (body
// b in block b % F2D_CLUSTER, slot b / F2D_CLUSTER) for the whole launch, and
// the stages are separated by the hardware cluster barrier, so a colour stage
// costs shared-memory round trips instead of L2 round trips and a grid-wide
// barrier. Constraint rows stream from L2; a colour's constraint k is always
// handled by the same thread, which therefore reads back its own impulses.
// ---------------------------------------------------------------------------
#define CLUSTER_THREADS 512
#define CLUSTER_SOLVER_MAX_BODIES 20000

__device__ __forceinline__ void integrate_velocity_smem( const DWorld& w, int b, float4& v4, const SolveParams& p )
{
	float4 m = w.massv[b];
	float4 dmp = w.damp[b];
	float4 f = w.force[b];
	float h = p.h;
	float maxLinearSpeedSq = p.maxLinearSpeed * p.maxLinearSpeed;
	float maxAngularSpeedSq = p.maxAngularSpeed * p.maxAngularSpeed;
	fv2 v = mk( v4.x, v4.y );
	float wv = v4.z;
	float linearDamping = 1.0f / ( 1.0f + h * dmp.x );
	float angularDamping = 1.0f / ( 1.0f + h * dmp.y );
	float gravityScale = m.x > 0.0f ? dmp.z : 0.0f;
	fv2 g = p.gravity;
	if ( w.subCount > 0 )
	{
		float2 gb = w.bodyGravity[b];
		g = mk( gb.x, gb.y );
	}
	fv2 lvd = vadd( vscale( h * m.x, mk( f.x, f.y ) ), vscale( h * gravityScale, g ) );
	float avd = h * m.y * f.z;
	v = vmuladd( lvd, linearDamping, v );
	wv = avd + angularDamping * wv;
	int flags = w.bflags[b];
	bool capped = false;
	if ( vdot( v, v ) > maxLinearSpeedSq )
	{
		float ratio = p.maxLinearSpeed / vlen( v );
		v = vscale( ratio, v );
		capped = true;
	}
	if ( wv * wv > maxAngularSpeedSq && ( flags & BF_FAST_ROT ) == 0 )
	{
		float ratio = p.maxAngularSpeed / fabs_s( wv );
		wv *= ratio;
		capped = true;
	}
	if ( capped )
		w.bflags[b] = flags | BF_SPEED_CAPPED;
	v4 = make_float4( v.x, v.y, wv, 0.0f );
}

__global__ void __launch_bounds__( CLUSTER_THREADS ) k_solve_cluster( DWorld w, SolveParams p, const int* jointSlots,
																	  const int* jointStart )
{
	extern __shared__ float4 sbody[]; // per slot: vel, delta
	__shared__ int sStart[F2D_COLORS], sCount[F2D_COLORS], sJStart[F2D_OVERFLOW + 1];
	cooperative_groups::cluster_group cl = cooperative_groups::this_cluster();
	const int rank = (int)cl.block_rank();
	if ( threadIdx.x < F2D_COLORS )
	{
		sStart[threadIdx.x] = w.sc->colorStart[threadIdx.x];
		sCount[threadIdx.x] = w.sc->colorCount[threadIdx.x];
	}
	if ( threadIdx.x <= F2D_OVERFLOW )
		sJStart[threadIdx.x] = jointStart[threadIdx.x];
	const int nb = w.bodyCount;
	const int slots = ( nb + F2D_CLUSTER - 1 ) / F2D_CLUSTER;
	for ( int sl = threadIdx.x; sl < slots; sl += blockDim.x )
	{
		int b = sl * F2D_CLUSTER + rank;
		if ( b < nb )
		{
			sbody[2 * sl] = __ldcg( w.vel + b );
			sbody[2 * sl + 1] = __ldcg( w.delta + b );
		}
	}
	cl.sync();

	const int stride = F2D_CLUSTER * blockDim.x;
	const int tid = rank * blockDim.x + threadIdx.x;
	const CBodies cb = { (unsigned)__cvta_generic_to_shared( sbody ) };
	const int novf = w.sc->overflowCount;
	const int novfJ = w.sc->overflowJointCount;
	const int nColour = w.sc->touchingCount - novf;
	const bool serialStage = novf > 0 || novfJ > 0;
	unsigned activeMask = 0;
	for ( int c = 0; c < F2D_OVERFLOW; ++c )
		if ( sCount[c] > 0 || sJStart[c + 1] > sJStart[c] )
			activeMask |= 1u << c;
	// block 0 of the cluster solves the overflow constraints, level by level
	__shared__ int sLevelStart[OVF_MAX_LEVELS + 1];
	__shared__ int sOrder[OVF_SMEM_ITEMS];
	OvfPlan plan = {};
	if ( serialStage && rank == 0 )
		plan = ovf_schedule( w, novf + novfJ <= OVF_SMEM_ITEMS ? sOrder : w.ovfOrder, sLevelStart );
	// colour slot r = threadIdx.x * F2D_CLUSTER + rank (+ stride ...) belongs to
	// this thread; the first one stays in registers for the whole launch
	const int r0 = threadIdx.x * F2D_CLUSTER + rank;
	Lane L0;
	int col0 = -1;
	if ( r0 < nColour )
	{
		int k0 = novf + r0;
		lane_load( w, k0, L0 );
		for ( int c = 0; c < F2D_OVERFLOW; ++c )
			if ( k0 >= sStart[c] && k0 < sStart[c] + sCount[c] )
				col0 = c;
	}

	for ( int sub = 0; sub < p.subSteps; ++sub )
	{
		for ( int sl = threadIdx.x; sl < slots; sl += blockDim.x )
		{
			int b = sl * F2D_CLUSTER + rank;
			if ( b < nb && body_awake( w.bflags[b] ) )
				integrate_velocity_smem( w, b, sbody[2 * sl], p );
		}
		cl.sync();
		for ( int kind = 0; kind < 3; ++kind )
		{
			if ( kind == 2 )
			{
				// integrate positions (solver.c:182-200)
				for ( int sl = threadIdx.x; sl < slots; sl += blockDim.x )
				{
					int b = sl * F2D_CLUSTER + rank;
					if ( b >= nb || !body_awake( w.bflags[b] ) )
						continue;
					float4 v = sbody[2 * sl];
					float4 d = sbody[2 * sl + 1];
					frot dq;
					dq.c = d.z;
					dq.s = d.w;
					dq = rintegrate( dq, p.h * v.z );
					fv2 dp = vmuladd( mk( d.x, d.y ), p.h, mk( v.x, v.y ) );
					sbody[2 * sl + 1] = make_float4( dp.x, dp.y, dq.c, dq.s );
				}
				cl.sync();
			}
			if ( serialStage )
			{
				if ( rank == 0 )
					ovf_stage( w, cb, plan, sLevelStart, kind, p );
				cl.sync();
			}
			for ( int c = 0; c < F2D_OVERFLOW; ++c )
			{
				if ( ( activeMask & ( 1u << c ) ) == 0 )
					continue;
				joint_colour_stage( w, cb, c, kind, p, tid, stride, jointSlots, sJStart );
				if ( col0 == c )
					lane_op( cb, L0, kind, p );
				colour_lanes_extra( w, cb, c, sStart, sCount, novf, tid, stride, kind, p );
				cl.sync();
			}
		}
	}
	// restitution: overflow then colours (solver.c:1103-1117)
	if ( novf > 0 )
	{
		if ( rank == 0 )
			ovf_stage( w, cb, plan, sLevelStart, 3, p );
		cl.sync();
	}
	for ( int c = 0; c < F2D_OVERFLOW; ++c )
	{
		if ( sCount[c] == 0 )
			continue;
		if ( col0 == c )
			lane_op( cb, L0, 3, p );
		colour_lanes_extra( w, cb, c, sStart, sCount, novf, tid, stride, 3, p );
		cl.sync();
	}
	// body rows back to the device, impulses into the manifolds
	for ( int sl = threadIdx.x; sl < slots; sl += blockDim.x )
	{
		int b = sl * F2D_CLUSTER + rank;
		if ( b < nb )
		{
			__stcg( w.vel + b, sbody[2 * sl] );
			__stcg( w.delta + b, sbody[2 * sl + 1] );
		}
	}
	for ( int k = tid; k < novf; k += stride )
		store_manifold_global( w, k, false );
	if ( col0 >= 0 )
		store_manifold( w, novf + r0, L0.imp, L0.tot, L0.misc.w, L0.pt[0].w, L0.pt[1].w,
						__float_as_int( L0.sf.w ), true );
	for ( int k = novf + stride + tid; k < novf + nColour; k += stride )
		store_manifold_global( w, k, true );
	// no block leaves while another may still address its shared memory
	cl.sync();
}

// Largest body count the cluster solver takes on this device (0 when a
// cluster of F2D_CLUSTER blocks with that much shared memory cannot run).
int solver_cluster_capacity()
{
	int dev = 0, optin = 0;
	cudaGetDevice( &dev );
	cudaDeviceGetAttribute( &optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev );
	cudaFuncAttributes fa = {};
	if ( cudaFuncGetAttributes( &fa, k_solve_cluster ) != cudaSuccess )
	{
		cudaGetLastError();
		return 0;
	}
	int dyn = optin - (int)fa.sharedSizeBytes - 256; // less the static shared memory and a margin
	if ( dyn < 32 * 64 )
		return 0;
	if ( cudaFuncSetAttribute( k_solve_cluster, cudaFuncAttributeNonPortableClusterSizeAllowed, 1 ) != cudaSuccess ||
		 cudaFuncSetAttribute( k_solve_cluster, cudaFuncAttributeMaxDynamicSharedMemorySize, dyn ) != cudaSuccess )
	{
		cudaGetLastError();
		return 0;
	}
	cudaLaunchConfig_t cfg = {};
	cfg.gridDim = dim3( F2D_CLUSTER );
	cfg.blockDim = dim3( CLUSTER_THREADS );
	cfg.dynamicSmemBytes = (size_t)dyn;
	cudaLaunchAttribute attr;
	attr.id = cudaLaunchAttributeClusterDimension;
	attr.val.clusterDim.x = F2D_CLUSTER;
	attr.val.clusterDim.y = 1;
	attr.val.clusterDim.z = 1;
	cfg.attrs = &attr;
	cfg.numAttrs = 1;
	int clusters = 0;
	if ( cudaOccupancyMaxActiveClusters( &clusters, k_solve_cluster, &cfg ) != cudaSuccess || clusters < 1 )
	{
		cudaGetLastError();
		return 0;
	}
	return ( dyn / 32 ) * F2D_CLUSTER;
}

// ---------------------------------------------------------------------------
// host driver
// ---------------------------------------------------------------------------
// Co-resident grid of the grid-wide solver: one block of 512 threads or two
// of 256 per SM (the cooperative launch checks co-residency).
template <int THREADS> static int grid_blocks( int perSMWanted )
{
	int perSM = 0;
	cudaOccupancyMaxActiveBlocksPerMultiprocessor( &perSM, k_solve<THREADS>, THREADS, 0 );
	int dev = 0;
	cudaGetDevice( &dev );
	int sms = 0;
	cudaDeviceGetAttribute( &sms, cudaDevAttrMultiProcessorCount, dev );
	if ( perSM < 1 )
		return 0;
	return sms * ( perSM < perSMWanted ? perSM : perSMWanted );
}

int solver_max_blocks( int threads )
{
	return threads == 256 ? grid_blocks<256>( 2 ) : grid_blocks<512>( 1 );
}

void launch_solver( DWorld& w, StepScratch& s, cudaStream_t st, float dt, int subSteps )
{
	SolveParams p;
	p.dt = dt;
	p.inv_dt = 1.0f / dt;
	p.h = dt / (float)subSteps;
	p.inv_h = (float)subSteps * p.inv_dt;
	float contactHertz = fmin_s( w.contactHertz, 0.125f * p.inv_h );
	p.contactSoft = make_soft( contactHertz, w.contactDampingRatio, p.h );
	p.staticSoft = make_soft( 2.0f * contactHertz, w.contactDampingRatio, p.h );
	float contactSpeed = w.maxContactPushSpeed / p.staticSoft.massScale;
	p.minBiasVel = -contactSpeed;
	p.pushout = w.maxContactPushSpeed;
	float jointHertz = fmin_s( w.jointHertz, 0.25f * p.inv_h );
	p.jointSoft = make_soft( jointHertz, w.jointDampingRatio, p.h );
	p.restitutionThreshold = w.restitutionThreshold;
	p.maxLinearSpeed = w.maxLinearSpeed;
	p.maxAngularSpeed = F2D_MAX_ROTATION * p.inv_dt;
	p.gravity = w.gravity;
	p.subSteps = subSteps;
	p.enableWarmStarting = w.enableWarmStarting;

	int* fill = s.tmpA; // F2D_COLORS ints
	k_zero_ints<<<1, 32, 0, st>>>( fill, F2D_COLORS );
	k_count_colors<<<grid_for( w.contactCap ), 256, 0, st>>>( w, fill );
	k_color_offsets<<<1, 1, 0, st>>>( w, fill );
	k_fill_slots<<<grid_for( w.contactCap ), 256, 0, st>>>( w, fill );
	k_prepare_contacts<<<grid_for( w.contactCap ), 256, 0, st>>>( w, p );
	if ( w.learnMode & 2 )
		launch_learned_warm_start( w, st );
	launch_prepare_joints( w, s, st, p.h, p.inv_h, p.jointSoft );

	int* jointSlots = s.tmpB;
	int* jointStart = s.tmpB + w.jointCap;
	void* args[] = { &w, &p, &jointSlots, &jointStart };
	// Small worlds solve on one cluster (all stages in distributed shared
	// memory and under the hardware cluster barrier); beyond about 2e4
	// bodies the cluster's 16 SMs no longer hold the constraints in registers
	// and the grid-wide solver is faster (measured: pyramid 0.11 vs 0.17 ms,
	// 25k pile equal, 100k pile 0.75 vs 0.26 ms).
	bool useCluster = s.clusterCapacity > 0 && w.bodyCount <= s.clusterCapacity &&
					  ( s.solverVariant == SOLVER_CLUSTER ||
						( s.solverVariant == SOLVER_AUTO && w.bodyCount <= CLUSTER_SOLVER_MAX_BODIES ) );
	if ( useCluster )
	{
		int slots = ( w.bodyCount + F2D_CLUSTER - 1 ) / F2D_CLUSTER;
		cudaLaunchConfig_t cfg = {};
		cfg.gridDim = dim3( F2D_CLUSTER );
		cfg.blockDim = dim3( CLUSTER_THREADS );
		cfg.dynamicSmemBytes = (size_t)( slots > 0 ? slots : 1 ) * 32;
		cfg.stream = st;
		cudaLaunchAttribute attr;
		attr.id = cudaLaunchAttributeClusterDimension;
		attr.val.clusterDim.x = F2D_CLUSTER;
		attr.val.clusterDim.y = 1;
		attr.val.clusterDim.z = 1;
		cfg.attrs = &attr;
		cfg.numAttrs = 1;
		if ( s.evSolveStart )
			cudaEventRecord( s.evSolveStart, st );
		cudaLaunchKernelEx( &cfg, k_solve_cluster, w, p, (const int*)jointSlots, (const int*)jointStart );
		return;
	}
	cudaMemsetAsync( &w.sc->barrierCount, 0, sizeof( unsigned ), st );
	if ( s.evSolveStart )
		cudaEventRecord( s.evSolveStart, st );
	if ( s.solverVariant == SOLVER_GRID256 && s.solverBlocks256 > 0 )
		cudaLaunchCooperativeKernel( (void*)k_solve<256>, dim3( s.solverBlocks256 ), dim3( 256 ), args, 0, st );
	else
		cudaLaunchCooperativeKernel( (void*)k_solve<512>, dim3( s.solverBlocks ), dim3( 512 ), args, 0, st );
}
