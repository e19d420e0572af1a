// Body finalisation after the solver: transforms, sleep velocity, fast-body
// detection and continuous collision against static shapes, shape AABB
// refresh with fat-AABB enlargement (which feeds the next step's pair
// search), move and hit events. Reference: packages/forge2d/third_party/
// box2d/src/solver.c:390-541 (b2SolveContinuous), :543-726
// (b2FinalizeBodiesTask), :1758-1913 (hit events, enlarged proxies).
#include "dnarrow.cuh"
#include "dtoi.cuh"
#include "dtree.cuh"
#include "dworld.cuh"
#include "kernels.cuh"

__device__ __forceinline__ bool awake_flags( int f )
{
	return ( f & ( BF_USED | BF_ENABLED | BF_ASLEEP ) ) == ( BF_USED | BF_ENABLED ) && body_type( f ) != 0;
}

__device__ __forceinline__ fbox shape_aabb( const float4* g, int type, fxf xf )
{
	float4 g0 = g[0];
	float4 g1 = g[1];
	fbox b;
	if ( type == ST_CIRCLE )
	{
		fv2 p = xpoint( xf, mk( g0.x, g0.y ) );
		float r = g1.x;
		b.lo = mk( p.x - r, p.y - r );
		b.hi = mk( p.x + r, p.y + r );
		return b;
	}
	if ( type == ST_CAPSULE || type == ST_SEGMENT || type == ST_CHAIN )
	{
		fv2 v1 = xpoint( xf, mk( g0.x, g0.y ) );
		fv2 v2 = xpoint( xf, mk( g0.z, g0.w ) );
		b.lo = vmin2( v1, v2 );
		b.hi = vmax2( v1, v2 );
		if ( type == ST_CAPSULE )
		{
			fv2 r = mk( g1.x, g1.x );
			b.lo = vsub( b.lo, r );
			b.hi = vadd( b.hi, r );
		}
		return b;
	}
	int count = __float_as_int( g1.y );
	float4 v01 = g[2];
	fv2 lo = xpoint( xf, mk( v01.x, v01.y ) );
	fv2 hi = lo;
	for ( int i = 1; i < count; ++i )
	{
		float4 vv = g[2 + ( i >> 1 )];
		fv2 v = ( i & 1 ) ? mk( vv.z, vv.w ) : mk( vv.x, vv.y );
		v = xpoint( xf, v );
		lo = vmin2( lo, v );
		hi = vmax2( hi, v );
	}
	fv2 r = mk( g1.x, g1.x );
	b.lo = vsub( lo, r );
	b.hi = vadd( hi, r );
	return b;
}

__global__ void k_finalize( DWorld w, float dt, float inv_dt )
{
	int n = w.bodyCount;
	for ( int b = blockIdx.x * blockDim.x + threadIdx.x; b < n; b += gridDim.x * blockDim.x )
	{
		int flags = w.bflags[b];
		if ( !awake_flags( flags ) )
			continue;
		float4 v4 = w.vel[b];
		float4 d = w.delta[b];
		float2 c2 = w.center[b];
		float4 x4 = w.xf[b];
		float4 mv = w.massv[b];
		float4 dm = w.damp[b];
		float4 fo = w.force[b];
		fv2 v = mk( v4.x, v4.y );
		float wv = v4.z;
		fv2 center = vadd( mk( c2.x, c2.y ), mk( d.x, d.y ) );
		frot q;
		q.c = x4.z;
		q.s = x4.w;
		frot dq;
		dq.c = d.z;
		dq.s = d.w;
		q = rnormalize( rmul( dq, q ) );
		float maxVelocity = vlen( v ) + fabs_s( wv ) * mv.w;
		float maxDeltaPosition = vlen( mk( d.x, d.y ) ) + fabs_s( dq.s ) * mv.w;
		float positionSleepFactor = 0.5f;
		float sleepVelocity = fmax_s( maxVelocity, positionSleepFactor * inv_dt * maxDeltaPosition );
		w.delta[b] = make_float4( 0.0f, 0.0f, 1.0f, 0.0f );
		float2 lc = w.localCenter[b];
		fv2 p = vsub( center, rrot( q, mk( lc.x, lc.y ) ) );
		w.center[b] = make_float2( center.x, center.y );
		w.xf[b] = make_float4( p.x, p.y, q.c, q.s );
		w.moveEvXf[b] = make_float4( p.x, p.y, q.c, q.s );
		float sleepTime = fo.w;
		flags &= ~( BF_SPEED_CAPPED | BF_IS_FAST );
		bool isFast = false;
		if ( w.enableSleep == 0 || ( flags & BF_ENABLE_SLEEP ) == 0 || sleepVelocity > dm.w )
		{
			sleepTime = 0.0f;
			if ( body_type( flags ) == 2 && w.enableContinuous && maxVelocity * dt > 0.5f * mv.z )
			{
				isFast = true;
				flags |= BF_IS_FAST;
				int slot = atomicAdd( &w.sc->fastCount, 1 );
				w.fastBodies[slot] = b;
			}
			else
				w.sweep0[b] = make_float4( center.x, center.y, q.c, q.s );
		}
		else
		{
			w.sweep0[b] = make_float4( center.x, center.y, q.c, q.s );
			sleepTime += dt;
		}
		w.force[b] = make_float4( 0.0f, 0.0f, 0.0f, sleepTime );
		w.bflags[b] = flags;
		if ( isFast )
			continue; // shapes are refreshed by the continuous kernel
		fxf xf;
		xf.p = p;
		xf.q = q;
		for ( int s = w.headShape[b], guard = 0; s != F2D_NULL && guard < ( 1 << 20 ); s = w.nextShape[s], ++guard )
		{
			int sf = w.sflags[s];
			fbox aabb = shape_aabb( w.geom + (size_t)s * GEOM_F4, shape_type( sf ), xf );
			aabb = box_grow( aabb, F2D_SPECULATIVE );
			w.aabb[s] = box_to4( aabb );
			fbox fat = box_from4( w.fat[s] );
			if ( !box_contains( fat, aabb ) )
			{
				w.fat[s] = box_to4( box_grow( aabb, F2D_AABB_MARGIN ) );
				w.sflags[s] = sf | SF_ENLARGED;
			}
		}
	}
}

__device__ __forceinline__ DProxy make_proxy( const float4* g, int type )
{
	DProxy p;
	float4 g0 = g[0], g1 = g[1];
	if ( type == ST_CIRCLE )
	{
		p.p[0] = mk( g0.x, g0.y );
		p.count = 1;
		p.radius = g1.x;
	}
	else if ( type == ST_CAPSULE || type == ST_SEGMENT || type == ST_CHAIN )
	{
		p.p[0] = mk( g0.x, g0.y );
		p.p[1] = mk( g0.z, g0.w );
		p.count = 2;
		p.radius = type == ST_CAPSULE ? g1.x : 0.0f;
	}
	else
	{
		int count = __float_as_int( g1.y );
		for ( int i = 0; i < 4; ++i )
		{
			float4 v = g[2 + i];
			p.p[2 * i] = mk( v.x, v.y );
			p.p[2 * i + 1] = mk( v.z, v.w );
		}
		p.count = count;
		p.radius = g1.x;
	}
	return p;
}

// min extent of one shape about a centre (shape.c:720-790)
__device__ __forceinline__ float shape_min_extent( const float4* g, int type )
{
	float4 g1 = g[1];
	if ( type == ST_CIRCLE || type == ST_CAPSULE )
		return g1.x;
	if ( type == ST_SEGMENT || type == ST_CHAIN )
		return 0.0f;
	int count = __float_as_int( g1.y );
	fv2 centroid = mk( g[0].x, g[0].y );
	float mn = F2D_HUGE;
	for ( int i = 0; i < count; ++i )
	{
		float4 vv = g[2 + ( i >> 1 )];
		float4 nn = g[6 + ( i >> 1 )];
		fv2 v = ( i & 1 ) ? mk( vv.z, vv.w ) : mk( vv.x, vv.y );
		fv2 nrm = ( i & 1 ) ? mk( nn.z, nn.w ) : mk( nn.x, nn.y );
		float planeOffset = vdot( nrm, vsub( v, centroid ) );
		mn = fmin_s( mn, planeOffset );
	}
	return mn + g1.x;
}

__device__ __forceinline__ bool filters_collide( const DWorld& w, int a, int b )
{
	int ga = w.group[a], gb = w.group[b];
	if ( ga == gb && ga != 0 )
		return ga > 0;
	return ( w.mask[a] & w.cat[b] ) != 0ull && ( w.cat[a] & w.mask[b] ) != 0ull;
}

__device__ __forceinline__ bool joint_allows( const DWorld& w, int ia, int ib )
{
	int key, other;
	if ( w.jointCountB[ia] < w.jointCountB[ib] )
	{
		key = w.headJoint[ia];
		other = ib;
	}
	else
	{
		key = w.headJoint[ib];
		other = ia;
	}
	for ( int guard = 0; key != F2D_NULL && guard < ( 1 << 20 ); ++guard )
	{
		int jid = key >> 1;
		int edge = key & 1;
		int2 jb = w.jbody[jid];
		int otherBody = edge == 0 ? jb.y : jb.x;
		if ( ( w.jflags[jid] & 0x10 ) == 0 && otherBody == other )
			return false;
		key = w.jnext[2 * jid + edge];
	}
	return true;
}

// solver.c:390-541: one thread per fast body; candidate static shapes are
// visited in shape-id order
#define CCD_LIST_MAX 64
#define CCD_CANDIDATES 32

__device__ __forceinline__ bool ccd_rejected( const DWorld& w, unsigned long long key )
{
	int lo = 0, hi = w.sc->cbReject;
	while ( lo < hi )
	{
		int mid = ( lo + hi ) >> 1;
		if ( w.cbReject[mid] < key )
			lo = mid + 1;
		else
			hi = mid;
	}
	return lo < w.sc->cbReject && w.cbReject[lo] == key;
}

// listOnly: with a custom filter, a first pass lists the (static shape,
// fast shape) candidates that reach the filter (solver.c:270-280) for the
// host and changes nothing; the second pass skips the ones it rejected.
__global__ void k_continuous( DWorld w, int listOnly )
{
	int n = w.sc->fastCount;
	for ( int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x )
	{
		int b = w.fastBodies[i];
		float4 s0 = w.sweep0[b];
		float2 c2 = w.center[b];
		float4 x4 = w.xf[b];
		float2 lc = w.localCenter[b];
		DSweep sweep;
		sweep.localCenter = mk( lc.x, lc.y );
		sweep.c1 = mk( s0.x, s0.y );
		sweep.c2 = mk( c2.x, c2.y );
		sweep.q1.c = s0.z;
		sweep.q1.s = s0.w;
		sweep.q2.c = x4.z;
		sweep.q2.s = x4.w;
		fxf xf1, xf2;
		xf1.q = sweep.q1;
		xf1.p = vsub( sweep.c1, rrot( sweep.q1, sweep.localCenter ) );
		xf2.q = sweep.q2;
		xf2.p = vsub( sweep.c2, rrot( sweep.q2, sweep.localCenter ) );
		float minExtent = w.massv[b].z;
		float fraction = 1.0f;
		for ( int fs = w.headShape[b], guard = 0; fs != F2D_NULL && guard < ( 1 << 20 ); fs = w.nextShape[fs], ++guard )
		{
			int sff = w.sflags[fs];
			int tf = shape_type( sff );
			const float4* gf = w.geom + (size_t)fs * GEOM_F4;
			fbox box1 = box_from4( w.aabb[fs] );
			fbox box2 = shape_aabb( gf, tf, xf2 );
			fbox box = box_union( box1, box2 );
			if ( !listOnly )
				w.aabb[fs] = box_to4( box2 );
			if ( sff & SF_SENSOR )
				continue;
			float4 gf1 = gf[1];
			fv2 centroid1 = xpoint( xf1, mk( gf1.z, gf1.w ) );
			fv2 centroid2 = xpoint( xf2, mk( gf1.z, gf1.w ) );
			// b2ContinuousQueryCallback (solver.c:196-388) for one static shape
			auto consider = [&]( int ss ) {
				int sfs = w.sflags[ss];
				if ( ( sfs & SF_USED ) == 0 )
					return;
				// the static tree's query skips categories of zero
				if ( w.cat[ss] == 0ull || !box_overlaps( box_from4( w.fat[ss] ), box ) )
					return;
				int sb = w.shapeBody[ss];
				if ( ss == fs || sb == b || ( sfs & SF_SENSOR ) ||
					 ( w.subCount > 0 && w.shapeSub[ss] != w.shapeSub[fs] ) )
					return;
				if ( !filters_collide( w, fs, ss ) )
					return;
				if ( w.bflags[sb] & BF_BULLET )
					return;
				if ( !joint_allows( w, b, sb ) )
					return;
				if ( w.callbacks & 1 )
				{
					unsigned long long key = ( (unsigned long long)ss << 32 ) | (unsigned)fs;
					if ( listOnly )
					{
						int slot = atomicAdd( &w.sc->cbList, 1 );
						if ( slot < w.cbCap )
							w.cbList[slot] = key;
						else
							atomicOr( &w.sc->error, ERR_EVENT_CAPACITY );
						return;
					}
					if ( ccd_rejected( w, key ) )
						return;
				}
				const float4* gs = w.geom + (size_t)ss * GEOM_F4;
				// solver.c:283-304: no pausing on chain segment junctions
				if ( shape_type( sfs ) == ST_CHAIN )
				{
					float4 st = w.xf[sb];
					fxf t;
					t.p = mk( st.x, st.y );
					t.q.c = st.z;
					t.q.s = st.w;
					float4 s0g = gs[0];
					fv2 p1 = xpoint( t, mk( s0g.x, s0g.y ) );
					fv2 p2 = xpoint( t, mk( s0g.z, s0g.w ) );
					float len;
					fv2 e = vlen_norm( &len, vsub( p2, p1 ) );
					if ( len > F2D_LINEAR_SLOP )
					{
						float offset1 = vcross( vsub( centroid1, p1 ), e );
						float offset2 = vcross( vsub( centroid2, p1 ), e );
						const float allowedFraction = 0.25f;
						if ( offset1 < 0.0f || offset1 - offset2 < allowedFraction * minExtent )
							return;
					}
				}
				DProxy pa = make_proxy( gs, shape_type( sfs ) );
				DProxy pb = make_proxy( gf, tf );
				float4 ss0 = w.sweep0[sb];
				float2 sc2 = w.center[sb];
				float4 sx4 = w.xf[sb];
				float2 slc = w.localCenter[sb];
				DSweep sa;
				sa.localCenter = mk( slc.x, slc.y );
				sa.c1 = mk( ss0.x, ss0.y );
				sa.c2 = mk( sc2.x, sc2.y );
				sa.q1.c = ss0.z;
				sa.q1.s = ss0.w;
				sa.q2.c = sx4.z;
				sa.q2.s = sx4.w;
				float f = time_of_impact( pa, pb, sa, sweep, fraction );
				if ( 0.0f < f && f < fraction )
					fraction = f;
				else if ( 0.0f == f )
				{
					float4 g0 = gf[0], g1 = gf[1];
					fv2 centroid = tf == ST_CIRCLE ? mk( g0.x, g0.y )
						: ( tf == ST_POLYGON ? mk( g0.x, g0.y ) : vlerp( mk( g0.x, g0.y ), mk( g0.z, g0.w ), 0.5f ) );
					(void)g1;
					float radius = 0.25f * shape_min_extent( gf, tf );
					DProxy pc;
					pc.p[0] = centroid;
					pc.count = 1;
					pc.radius = radius;
					f = time_of_impact( pa, pc, sa, sweep, fraction );
					if ( 0.0f < f && f < fraction )
						fraction = f;
				}
			};
			// candidates in the static tree's depth-first order (descending
			// left-to-right rank), as the reference's query meets them: the
			// static list (kept in that order) when it is short, else the
			// static leaves of the pair tree overlapping the sweep box
			bool scanList = w.staticCount <= CCD_LIST_MAX;
			int cand[CCD_CANDIDATES];
			int nc = 0;
			if ( !scanList )
			{
				bool overflow = false;
				bool done = tree_query( w, w.sc->treeLeafCount, box, [&]( int leaf ) {
					int ss = w.leafShape[leaf];
					if ( ( w.proxyKey[ss] & 3 ) != 0 )
						return;
					if ( nc == CCD_CANDIDATES )
					{
						overflow = true;
						return;
					}
					int k = nc++;
					int rs = w.pt[0].rank[w.proxyKey[ss] >> 2];
					while ( k > 0 && w.pt[0].rank[w.proxyKey[cand[k - 1]] >> 2] < rs )
					{
						cand[k] = cand[k - 1];
						k -= 1;
					}
					cand[k] = ss;
				} );
				scanList = overflow || !done;
			}
			if ( scanList )
			{
				for ( int k = 0; k < w.staticCount; ++k )
					consider( w.staticShapes[k] );
			}
			else
			{
				for ( int k = 0; k < nc; ++k )
					consider( cand[k] );
			}
		}
		if ( listOnly )
			continue;
		if ( fraction < 1.0f )
		{
			frot q = rnlerp( sweep.q1, sweep.q2, fraction );
			fv2 c = vlerp( sweep.c1, sweep.c2, fraction );
			fv2 origin = vsub( c, rrot( q, sweep.localCenter ) );
			w.xf[b] = make_float4( origin.x, origin.y, q.c, q.s );
			w.moveEvXf[b] = make_float4( origin.x, origin.y, q.c, q.s );
			w.center[b] = make_float2( c.x, c.y );
			w.sweep0[b] = make_float4( c.x, c.y, q.c, q.s );
			fxf t;
			t.p = origin;
			t.q = q;
			for ( int s = w.headShape[b], guard = 0; s != F2D_NULL && guard < ( 1 << 20 ); s = w.nextShape[s], ++guard )
			{
				int sf = w.sflags[s];
				fbox aabb = shape_aabb( w.geom + (size_t)s * GEOM_F4, shape_type( sf ), t );
				aabb = box_grow( aabb, F2D_SPECULATIVE );
				w.aabb[s] = box_to4( aabb );
				if ( !box_contains( box_from4( w.fat[s] ), aabb ) )
				{
					w.fat[s] = box_to4( box_grow( aabb, F2D_AABB_MARGIN ) );
					w.sflags[s] = sf | SF_ENLARGED;
				}
			}
		}
		else
		{
			w.sweep0[b] = make_float4( sweep.c2.x, sweep.c2.y, sweep.q2.c, sweep.q2.s );
			for ( int s = w.headShape[b], guard = 0; s != F2D_NULL && guard < ( 1 << 20 ); s = w.nextShape[s], ++guard )
			{
				int sf = w.sflags[s];
				fbox aabb = box_from4( w.aabb[s] );
				if ( !box_contains( box_from4( w.fat[s] ), aabb ) )
				{
					w.fat[s] = box_to4( box_grow( aabb, F2D_AABB_MARGIN ) );
					w.sflags[s] = sf | SF_ENLARGED;
				}
			}
		}
	}
}

// solver.c:1758-1818 hit events
__global__ void k_hit_events( DWorld w )
{
	int n = w.sc->touchingCount;
	for ( int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x )
	{
		int c = w.slotContact[k];
		if ( ( w.cflags[c] & CF_HIT_EVENT ) == 0 )
			continue;
		float4 mn = w.mnorm[c];
		int count = __float_as_int( mn.w );
		float approach = w.hitEventThreshold;
		bool hit = false;
		fv2 point = mk( 0.0f, 0.0f );
		for ( int j = 0; j < count; ++j )
		{
			float4 im = w.mpI[2 * c + j];
			float s = -im.w;
			if ( s > approach && im.z > 0.0f )
			{
				approach = s;
				float4 pb = w.mpB[2 * c + j];
				point = mk( pb.x, pb.y );
				hit = true;
			}
		}
		if ( hit )
		{
			int e = atomicAdd( &w.sc->hitCount, 1 );
			if ( e < w.eventCap )
			{
				int2 s = w.cshape[c];
				w.hitEvI[2 * e] = s.x;
				w.hitEvI[2 * e + 1] = s.y;
				float* o = w.hitEvF + 5 * e;
				o[0] = point.x;
				o[1] = point.y;
				o[2] = mn.x;
				o[3] = mn.y;
				o[4] = approach;
			}
		}
	}
}

__global__ void k_reset_step_counters( DWorld w )
{
	w.sc->hitCount = 0;
	w.sc->fastCount = 0;
	w.sc->newPointCount = 0;
	for ( int k = 0; k < 8; ++k )
		w.sc->npCount[k] = 0;
	int age = w.sc->orderAge;
	int period = w.sc->orderPeriod > 0 ? w.sc->orderPeriod : ORDER_REBUILD_PERIOD;
	int rebuild = ( w.sc->forceRebuild != 0 || age >= period - 1 ) ? 1 : 0;
	w.sc->rebuildOrder = rebuild;
	w.sc->orderAge = rebuild ? 0 : age + 1;
	w.sc->forceRebuild = 0;
}

void launch_finalize( DWorld& w, StepScratch& s, cudaStream_t st, float dt, HostHook ccdHook, void* hookContext )
{
	(void)s;
	if ( w.isl )
		launch_isl_split( w, st );
	k_finalize<<<grid_for( w.bodyCount ), 256, 0, st>>>( w, dt, 1.0f / dt );
	if ( ccdHook )
	{
		cudaMemsetAsync( &w.sc->cbList, 0, sizeof( int ), st );
		k_continuous<<<grid_for( w.bodyCount ), 64, 0, st>>>( w, 1 );
		ccdHook( hookContext );
	}
	k_continuous<<<grid_for( w.bodyCount ), 64, 0, st>>>( w, 0 );
	k_hit_events<<<grid_for( w.contactCap ), 256, 0, st>>>( w );
	// solver.c:1842-1905: enlarged proxies enter the move array of the next
	// step in awake order and grow their tree leaves
	launch_pt_moves( w, s, st );
	if ( w.isl )
		launch_isl_sleep( w, st, s.scanState );
}

void launch_reset_counters( DWorld& w, cudaStream_t st )
{
	k_reset_step_counters<<<1, 1, 0, st>>>( w );
}
