// Narrowphase of the world step: one thread per live contact refreshes its
// manifold, carries warm-start impulses over by point id and raises the
// state-change flags, as b2CollideTask + b2UpdateContact do
// (packages/forge2d/third_party/box2d/src/world.c:357-445,
// contact.c:472-600). The contacts that changed state are then compacted in
// contact-id order, the order in which the reference applies them serially
// (world.c:586-686).
#include "dnarrow.cuh"
#include "dscan.cuh"
#include "dsort.cuh"
#include "dworld.cuh"
#include "kernels.cuh"

#define NP_THREADS 128

__device__ __forceinline__ float shape_radius( int type, const float4* g )
{
	return ( type == ST_CIRCLE || type == ST_CAPSULE || type == ST_POLYGON ) ? g[1].x : 0.0f;
}

// Manifold class of a contact (shape A's type >= shape B's type, the
// registry order of contact.c:151-205).
__device__ __forceinline__ int manifold_class( int ta, int tb )
{
	if ( ta == ST_CIRCLE && tb == ST_CIRCLE )
		return 0;
	if ( ( ta == ST_CAPSULE || ta == ST_SEGMENT ) && tb == ST_CIRCLE )
		return 1;
	if ( ( ta == ST_CAPSULE || ta == ST_SEGMENT ) && tb == ST_CAPSULE )
		return 2;
	if ( ta == ST_POLYGON && tb == ST_CIRCLE )
		return 3;
	return 4;
}

// The manifold function compute_manifold selects for the class, called
// directly so that each class kernel holds only its own path.
template <int CLS>
__device__ __forceinline__ DManifold class_manifold( const DGeom& a, fxf xfA, const DGeom& b, fxf xfB, DCache& cache )
{
	if ( CLS == 0 )
		return collide_circles( a.c1, a.radius, xfA, b.c1, b.radius, xfB );
	if ( CLS == 1 )
		return collide_capsule_circle( a.c1, a.c2, a.type == ST_SEGMENT ? 0.0f : a.radius, xfA, b.c1, b.radius, xfB );
	if ( CLS == 2 )
		return collide_capsules( a.c1, a.c2, a.type == ST_SEGMENT ? 0.0f : a.radius, xfA, b.c1, b.c2, b.radius, xfB );
	if ( CLS == 3 )
		return collide_polygon_circle( a.poly, xfA, b.c1, b.radius, xfB );
	return compute_manifold( a, xfA, b, xfB, cache );
}

// Fat-AABB test of every live contact (b2CollideTask's disjoint check); the
// overlapping ones are listed by manifold class so that every warp of a
// class kernel runs one manifold function. Bucket order is irrelevant: each
// contact's update depends on that contact alone.
__global__ void k_np_classify( DWorld w )
{
	const int n = w.sc->contactIdCount;
	const unsigned lane = threadIdx.x & 31u;
	// grid-stride with a block-uniform trip count: the append is warp-collective
	for ( int base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x )
	{
		int c = base + threadIdx.x;
		int cls = -1;
		if ( c < n )
		{
			int flags = w.cflags[c];
			// contacts outside the awake set are not collided (b2Collide walks
			// the awake contact array)
			if ( ( flags & ( CF_USED | CF_INACTIVE ) ) == CF_USED )
			{
				int2 sh = w.cshape[c];
				fbox fa = box_from4( w.fat[sh.x] );
				fbox fb = box_from4( w.fat[sh.y] );
				if ( !box_overlaps( fa, fb ) )
				{
					flags |= CF_DISJOINT;
					flags &= ~CF_SIM_TOUCHING;
					w.cflags[c] = flags;
				}
				else
					cls = manifold_class( shape_type( w.sflags[sh.x] ), shape_type( w.sflags[sh.y] ) );
			}
		}
		// warp-aggregated append per class
		unsigned peers = __match_any_sync( 0xffffffffu, cls );
		if ( cls >= 0 )
		{
			int leader = __ffs( peers ) - 1;
			int slot = 0;
			if ( (int)lane == leader )
				slot = atomicAdd( w.sc->npCount + cls, __popc( peers ) );
			slot = __shfl_sync( peers, slot, leader );
			int rank = __popc( peers & ( ( 1u << lane ) - 1u ) );
			w.npBucket[(size_t)cls * w.contactCap + slot + rank] = c;
		}
	}
}

__device__ __forceinline__ bool sorted_contains( const unsigned long long* keys, int n, unsigned long long key )
{
	int lo = 0, hi = n;
	while ( lo < hi )
	{
		int mid = ( lo + hi ) >> 1;
		if ( keys[mid] < key )
			lo = mid + 1;
		else
			hi = mid;
	}
	return lo < n && keys[lo] == key;
}

__device__ __forceinline__ fxf xf_of( float4 x )
{
	fxf t;
	t.p = mk( x.x, x.y );
	t.q.c = x.z;
	t.q.s = x.w;
	return t;
}

// Lists, for the host's pre-solve callback, every awake overlapping contact
// with pre-solve events whose new manifold has points, with that manifold
// as the callback sees it (20 floats laid out as f2d_manifold_view: anchors
// still relative to the body origins) and the two shape ids. The GJK cache is read, not written: the class kernels then
// compute the same manifold from the same cache.
__global__ void k_presolve_list( DWorld w )
{
	const int n = w.sc->contactIdCount;
	for ( int c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x )
	{
		int flags = w.cflags[c];
		if ( ( flags & ( CF_USED | CF_INACTIVE | CF_PRESOLVE ) ) != ( CF_USED | CF_PRESOLVE ) )
			continue;
		int2 sh = w.cshape[c];
		if ( !box_overlaps( box_from4( w.fat[sh.x] ), box_from4( w.fat[sh.y] ) ) )
			continue;
		int2 bd = w.cbody[c];
		fxf xfA = xf_of( w.xf[bd.x] ), xfB = xf_of( w.xf[bd.y] );
		int ta = shape_type( w.sflags[sh.x] ), tb = shape_type( w.sflags[sh.y] );
		DGeom A = load_geom( w.geom + (size_t)sh.x * GEOM_F4, ta );
		DGeom B = load_geom( w.geom + (size_t)sh.y * GEOM_F4, tb );
		DCache cache = unpack_cache( w.csimplex[c] );
		DManifold m = compute_manifold( A, xfA, B, xfB, cache );
		if ( m.count == 0 )
			continue;
		int slot = atomicAdd( &w.sc->cbList, 1 );
		if ( slot >= w.cbCap )
		{
			atomicOr( &w.sc->error, ERR_EVENT_CAPACITY );
			continue;
		}
		w.cbList[slot] = (unsigned long long)c;
		float* o = w.cbManifold + (size_t)slot * 22;
		o[20] = __int_as_float( sh.x );
		o[21] = __int_as_float( sh.y );
		o[0] = m.normal.x;
		o[1] = m.normal.y;
		o[2] = __int_as_float( m.count );
		o[3] = 0.0f;
		for ( int i = 0; i < 2; ++i )
		{
			const DPoint& p = m.p[i];
			float* q = o + 4 + 8 * i;
			q[0] = p.point.x;
			q[1] = p.point.y;
			q[2] = p.anchorA.x;
			q[3] = p.anchorA.y;
			q[4] = p.anchorB.x;
			q[5] = p.anchorB.y;
			q[6] = p.separation;
			q[7] = __int_as_float( (int)p.id );
		}
	}
}

// b2UpdateContact (contact.c:472-600) for the contacts of one class.
template <int CLS> __global__ void __launch_bounds__( NP_THREADS ) k_narrowphase( DWorld w )
{
	const int n = w.sc->npCount[CLS];
	const int* bucket = w.npBucket + (size_t)CLS * w.contactCap;
	for ( int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x )
	{
		int c = bucket[i];
		int flags = w.cflags[c];
		int2 sh = w.cshape[c];
		bool wasTouching = ( flags & CF_SIM_TOUCHING ) != 0;
		int2 bd = w.cbody[c];
		float4 ma = w.massv[bd.x], mb = w.massv[bd.y];
		w.cmass[c] = make_float4( ma.x, ma.y, mb.x, mb.y );
		float4 xa4 = w.xf[bd.x], xb4 = w.xf[bd.y];
		fxf xfA, xfB;
		xfA.p = mk( xa4.x, xa4.y );
		xfA.q.c = xa4.z;
		xfA.q.s = xa4.w;
		xfB.p = mk( xb4.x, xb4.y );
		xfB.q.c = xb4.z;
		xfB.q.s = xb4.w;
		float2 lca = w.localCenter[bd.x], lcb = w.localCenter[bd.y];
		fv2 offA = rrot( xfA.q, mk( lca.x, lca.y ) );
		fv2 offB = rrot( xfB.q, mk( lcb.x, lcb.y ) );
		int sfa = w.sflags[sh.x], sfb = w.sflags[sh.y];
		int ta = shape_type( sfa ), tb = shape_type( sfb );
		const float4* ga = w.geom + (size_t)sh.x * GEOM_F4;
		const float4* gb = w.geom + (size_t)sh.y * GEOM_F4;
		DGeom A = load_geom( ga, ta );
		DGeom B = load_geom( gb, tb );
		// the contact's GJK cache (chain segments against capsules and polygons)
		bool chain = CLS == 4 && ta == ST_CHAIN;
		DCache cache;
		cache.count = 0;
		if ( chain )
			cache = unpack_cache( w.csimplex[c] );
		DManifold m = class_manifold<CLS>( A, xfA, B, xfB, cache );
		if ( chain )
			w.csimplex[c] = pack_cache( cache );

		float4 mta = w.mat[sh.x], mtb = w.mat[sh.y];
		float friction = sqrtf( mta.x * mtb.x );
		float restitution = mta.y > mtb.y ? mta.y : mtb.y;
		float rolling = 0.0f;
		if ( mta.z > 0.0f || mtb.z > 0.0f )
		{
			float ra = shape_radius( ta, ga ), rb = shape_radius( tb, gb );
			float mr = fmax_s( ra, rb );
			rolling = fmax_s( mta.z, mtb.z ) * mr;
		}
		float tangentSpeed = mta.w + mtb.w;
		w.cmat[c] = make_float4( friction, restitution, rolling, tangentSpeed );

		int rawCount = m.count;
		int pointCount = rawCount;
		// contact.c:504-517: a pre-solve callback that returned false (the host
		// listed it in cbReject) disables the contact for this step
		if ( ( w.callbacks & 2 ) && ( flags & CF_PRESOLVE ) && rawCount > 0 &&
			 sorted_contains( w.cbReject, w.sc->cbReject, (unsigned long long)c ) )
			pointCount = 0;
		bool touching = pointCount > 0;
		if ( touching && ( ( sfa | sfb ) & SF_HIT_EVENTS ) )
			flags |= CF_HIT_EVENT;
		else
			flags &= ~CF_HIT_EVENT;

		// old manifold (ids and impulses)
		float4 oldN = w.mnorm[c];
		int oldCount = __float_as_int( oldN.w );
		unsigned oldId[2];
		float oldNI[2], oldTI[2];
		for ( int k = 0; k < 2; ++k )
		{
			oldId[k] = (unsigned)__float_as_int( w.mpB[2 * c + k].w ) & 0xffffu;
			float4 im = w.mpI[2 * c + k];
			oldNI[k] = im.x;
			oldTI[k] = im.y;
		}
		float rollingImpulse = pointCount > 0 ? oldN.z : 0.0f;
		fv2 normal = rawCount > 0 ? m.normal : mk( 0.0f, 0.0f );
		w.mnorm[c] = make_float4( normal.x, normal.y, rollingImpulse, __int_as_float( pointCount ) );
		for ( int i = 0; i < 2; ++i )
		{
			if ( i < pointCount )
			{
				DPoint p = m.p[i];
				fv2 anchorA = vsub( p.anchorA, offA );
				fv2 anchorB = vsub( p.anchorB, offB );
				float ni = 0.0f, ti = 0.0f;
				int persisted = 0;
				for ( int j = 0; j < oldCount; ++j )
				{
					if ( oldId[j] == p.id )
					{
						ni = oldNI[j];
						ti = oldTI[j];
						persisted = 1;
						break;
					}
				}
				w.mpA[2 * c + i] = make_float4( anchorA.x, anchorA.y, anchorB.x, anchorB.y );
				w.mpB[2 * c + i] = make_float4( p.point.x, p.point.y, p.separation,
												__int_as_float( (int)( p.id | ( persisted << 16 ) ) ) );
				w.mpI[2 * c + i] = make_float4( ni, ti, 0.0f, 0.0f );
			}
			else
			{
				// slot past pointCount: kept as the manifold function left it
				// (contact.c:472-560 replaces the whole manifold and touches
				// only the first pointCount points)
				DPoint p = m.p[i];
				w.mpA[2 * c + i] = make_float4( p.anchorA.x, p.anchorA.y, p.anchorB.x, p.anchorB.y );
				w.mpB[2 * c + i] = make_float4( p.point.x, p.point.y, p.separation, __int_as_float( (int)p.id ) );
				w.mpI[2 * c + i] = make_float4( 0.0f, 0.0f, 0.0f, 0.0f );
			}
		}
		if ( touching )
			flags |= CF_SIM_TOUCHING;
		else
			flags &= ~CF_SIM_TOUCHING;
		if ( touching && !wasTouching )
			flags |= CF_STARTED;
		else if ( !touching && wasTouching )
			flags |= CF_STOPPED;
		w.cflags[c] = flags;
	}
}

__global__ void k_op_flags( DWorld w, int* flags )
{
	int n = w.sc->contactIdCount;
	for ( int c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x )
	{
		int f = w.cflags[c];
		flags[c] = ( ( f & CF_USED ) && ( f & ( CF_DISJOINT | CF_STARTED | CF_STOPPED ) ) ) ? 1 : 0;
	}
}

__global__ void k_op_compact( DWorld w, const int* flags, const int* offs )
{
	int n = w.sc->contactIdCount;
	for ( int c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x )
	{
		if ( flags[c] == 0 )
			continue;
		int o = offs[c];
		if ( o >= w.opCap )
		{
			atomicOr( &w.sc->error, ERR_OP_CAPACITY );
			continue;
		}
		int f = w.cflags[c];
		w.opContact[o] = c;
		w.opKind[o] = ( f & CF_DISJOINT ) ? 0 : ( ( f & CF_STARTED ) ? 1 : 2 );
	}
}

__global__ void k_op_clamp( DWorld w )
{
	if ( w.sc->opCount > w.opCap )
		w.sc->opCount = w.opCap;
}

void launch_narrowphase( DWorld& w, StepScratch& s, cudaStream_t st, HostHook preSolveHook, void* hookContext )
{
	int g = ( w.contactCap + NP_THREADS - 1 ) / NP_THREADS;
	if ( g > F2D_SMS * 8 )
		g = F2D_SMS * 8;
	if ( preSolveHook )
	{
		// the callback runs between the listing and the manifold update
		cudaMemsetAsync( &w.sc->cbList, 0, sizeof( int ), st );
		k_presolve_list<<<g, NP_THREADS, 0, st>>>( w );
		preSolveHook( hookContext );
	}
	k_np_classify<<<grid_for( w.contactCap ), 256, 0, st>>>( w );
	// the classes update disjoint contacts: the polygon clipper and three
	// short classes run beside the first class, each on its own stream
	cudaStream_t cs[5] = { st, st, st, st, st };
	if ( s.side[0] )
	{
		cudaEventRecord( s.sideFork, st );
		for ( int k = 0; k < 4; ++k )
		{
			cudaStreamWaitEvent( s.side[k], s.sideFork, 0 );
			cs[4 - k] = s.side[k];
		}
	}
	k_narrowphase<4><<<g, NP_THREADS, 0, cs[4]>>>( w );
	k_narrowphase<3><<<g, NP_THREADS, 0, cs[3]>>>( w );
	k_narrowphase<2><<<g, NP_THREADS, 0, cs[2]>>>( w );
	k_narrowphase<1><<<g, NP_THREADS, 0, cs[1]>>>( w );
	k_narrowphase<0><<<g, NP_THREADS, 0, cs[0]>>>( w );
	if ( s.side[0] )
		for ( int k = 0; k < 4; ++k )
		{
			cudaEventRecord( s.sideJoin[k], s.side[k] );
			cudaStreamWaitEvent( st, s.sideJoin[k], 0 );
		}
	k_op_flags<<<grid_for( w.contactCap ), 256, 0, st>>>( w, s.tmpA );
	scan_lookback( s.tmpA, s.tmpB, &w.sc->contactIdCount, 0, w.contactCap, &w.sc->opCount, s.scanState, &w.sc->error,
				   st );
	k_op_compact<<<grid_for( w.contactCap ), 256, 0, st>>>( w, s.tmpA, s.tmpB );
	k_op_clamp<<<1, 1, 0, st>>>( w );
}
