// b2World_Explode (packages/forge2d/third_party/box2d/src/world.c:2640-2735)
// on the device: every shape of a dynamic body whose fat AABB meets the
// blast box (category against the mask) and lies within radius + falloff of
// the centre (GJK with radii) wakes its body and gets an impulse along the
// centre-to-closest-point direction, scaled by its projected perimeter
// (shape.c:655-703) and the falloff. A body's shapes apply in ascending
// shape id, sleeping sets wake in ascending shape id (the reference visits
// its dynamic tree's order; that order shows only for bodies with several
// shapes in the blast and for the order sleeping sets wake in).
#include "dtoi.cuh"
#include "dworld.cuh"
#include "kernels.cuh"

#include <climits>

struct Blast
{
	fv2 position;
	float radius, falloff, impulsePerLength;
	unsigned long long mask;
};

__device__ __forceinline__ DProxy blast_proxy( const float4* g, int type )
{
	DProxy p;
	float4 g0 = g[0], g1 = g[1];
	if ( type == ST_CIRCLE )
	{
		p.p[0] = mk( g0.x, g0.y );
		p.count = 1;
		p.radius = g1.x;
	}
	else if ( type == ST_POLYGON )
	{
		for ( int i = 0; i < 4; ++i )
		{
			float4 v = g[2 + i];
			p.p[2 * i] = mk( v.x, v.y );
			p.p[2 * i + 1] = mk( v.z, v.w );
		}
		p.count = __float_as_int( g1.y );
		p.radius = g1.x;
	}
	else
	{
		p.p[0] = mk( g0.x, g0.y );
		p.p[1] = mk( g0.z, g0.w );
		p.count = 2;
		p.radius = type == ST_CAPSULE ? g1.x : 0.0f;
	}
	return p;
}

// distance with radii (distance.c:592-603) and the closest point on the shape
__device__ __forceinline__ float blast_distance( const DWorld& w, int s, fxf xf, const Blast& bl, fv2& pointA )
{
	DProxy pa = blast_proxy( w.geom + (size_t)s * GEOM_F4, shape_type( w.sflags[s] ) );
	DProxy pb;
	pb.p[0] = bl.position;
	pb.count = 1;
	pb.radius = 0.0f;
	fxf identity;
	identity.p = mk( 0.0f, 0.0f );
	identity.q.c = 1.0f;
	identity.q.s = 0.0f;
	DCache cache;
	cache.count = 0;
	fv2 pointB, normal;
	pointA = mk( 0.0f, 0.0f );
	float d = gjk_distance( pa, pb, xf, identity, cache, &pointA, &pointB, &normal );
	if ( d > 0.1f * F2D_LINEAR_SLOP )
	{
		d = fmax_s( 0.0f, d - pa.radius - pb.radius );
		pointA = vmuladd( pointA, pa.radius, normal );
	}
	return d;
}

__device__ __forceinline__ fxf body_xform( const DWorld& w, int b )
{
	float4 x = w.xf[b];
	fxf t;
	t.p = mk( x.x, x.y );
	t.q.c = x.z;
	t.q.s = x.w;
	return t;
}

__device__ __forceinline__ bool blast_candidate( const DWorld& w, int s, const Blast& bl )
{
	int f = w.sflags[s];
	if ( ( f & ( SF_USED | SF_PROXY ) ) != ( SF_USED | SF_PROXY ) || ( w.proxyKey[s] & 3 ) != 2 )
		return false;
	if ( ( w.cat[s] & bl.mask ) == 0ull )
		return false;
	float e = bl.radius + bl.falloff;
	fbox box;
	box.lo = mk( bl.position.x - e, bl.position.y - e );
	box.hi = mk( bl.position.x + e, bl.position.y + e );
	return box_overlaps( box_from4( w.fat[s] ), box );
}

// hit[s] = 1 + the shape's left-to-right position in the dynamic tree for
// the shapes the blast reaches (the reference's query visits them in
// descending position, world.c:2746), else 0; byRank[position] = s
__global__ void k_explode_mark( DWorld w, Blast bl, int* hit, int* byRank )
{
	for ( int s = blockIdx.x * blockDim.x + threadIdx.x; s < w.shapeCount; s += gridDim.x * blockDim.x )
	{
		int h = 0;
		if ( blast_candidate( w, s, bl ) )
		{
			fv2 pA;
			if ( blast_distance( w, s, body_xform( w, w.shapeBody[s] ), bl, pA ) <= bl.radius + bl.falloff )
			{
				int r = tree_leaf_rank( w.pt[2], w.proxyKey[s] >> 2 );
				if ( r >= 0 && r < w.shapeCap )
				{
					h = r + 1;
					byRank[r] = s;
				}
			}
		}
		hit[s] = h;
	}
}

// shape.c:655-703 b2GetShapeProjectedPerimeter
__device__ __forceinline__ float projected_perimeter( const float4* g, int type, fv2 line )
{
	float4 g0 = g[0], g1 = g[1];
	if ( type == ST_CAPSULE )
	{
		fv2 axis = vsub( mk( g0.z, g0.w ), mk( g0.x, g0.y ) );
		return fabs_s( vdot( axis, line ) ) + 2.0f * g1.x;
	}
	if ( type == ST_CIRCLE )
		return 2.0f * g1.x;
	if ( type == ST_POLYGON )
	{
		int count = __float_as_int( g1.y );
		float lower = 0.0f, upper = 0.0f;
		for ( int i = 0; i < count; ++i )
		{
			float4 vv = g[2 + ( i >> 1 )];
			fv2 v = ( i & 1 ) ? mk( vv.z, vv.w ) : mk( vv.x, vv.y );
			float value = vdot( v, line );
			lower = i == 0 ? value : fmin_s( lower, value );
			upper = i == 0 ? value : fmax_s( upper, value );
		}
		return ( upper - lower ) + 2.0f * g1.x;
	}
	float value1 = vdot( mk( g0.x, g0.y ), line );
	float value2 = vdot( mk( g0.z, g0.w ), line );
	return fabs_s( value2 - value1 );
}

// one thread per body: its hit shapes in the query's order (descending
// tree position), so the impulses add up as the reference's do
__global__ void k_explode_apply( DWorld w, Blast bl, const int* hit )
{
	for ( int b = blockIdx.x * blockDim.x + threadIdx.x; b < w.bodyCount; b += gridDim.x * blockDim.x )
	{
		int bf = w.bflags[b];
		if ( ( bf & BF_USED ) == 0 || ( bf & BF_ENABLED ) == 0 || body_type( bf ) != 2 || ( bf & BF_ASLEEP ) )
			continue;
		fxf xf = body_xform( w, b );
		float4 v = w.vel[b];
		float4 mv = w.massv[b];
		float2 c = w.center[b];
		bool touched = false;
		int last = INT_MAX;
		for ( int guard = 0; guard < 4096; ++guard )
		{
			// next hit shape of this body below position `last`
			int next = -1, nextPos = 0;
			for ( int s = w.headShape[b], g2 = 0; s != F2D_NULL && g2 < 4096; s = w.nextShape[s], ++g2 )
				if ( hit[s] && hit[s] < last && hit[s] > nextPos )
				{
					next = s;
					nextPos = hit[s];
				}
			if ( next < 0 )
				break;
			last = nextPos;
			int s = next;
			fv2 pointA;
			float d = blast_distance( w, s, xf, bl, pointA );
			fv2 closestPoint = pointA;
			const float4* g = w.geom + (size_t)s * GEOM_F4;
			int type = shape_type( w.sflags[s] );
			if ( d == 0.0f )
			{
				float4 g1 = g[1];
				closestPoint = xpoint( xf, mk( g1.z, g1.w ) );
			}
			fv2 direction = vsub( closestPoint, bl.position );
			if ( vlen2( direction ) > 100.0f * FLT_EPSILON * FLT_EPSILON )
				direction = vnormalize( direction );
			else
				direction = mk( 1.0f, 0.0f );
			fv2 localLine = rinvrot( xf.q, vleft( direction ) );
			float perimeter = projected_perimeter( g, type, localLine );
			float scale = 1.0f;
			if ( d > bl.radius && bl.falloff > 0.0f )
				scale = fclamp_s( ( bl.radius + bl.falloff - d ) / bl.falloff, 0.0f, 1.0f );
			float magnitude = bl.impulsePerLength * perimeter * scale;
			fv2 impulse = vscale( magnitude, direction );
			fv2 lin = vmuladd( mk( v.x, v.y ), mv.x, impulse );
			v.x = lin.x;
			v.y = lin.y;
			v.z += mv.y * vcross( vsub( closestPoint, mk( c.x, c.y ) ), impulse );
			touched = true;
		}
		if ( touched )
			w.vel[b] = v;
	}
}

void launch_explode( DWorld& w, cudaStream_t st, int* hit, unsigned long long mask, float x, float y, float radius,
					 float falloff, float impulsePerLength )
{
	Blast bl;
	bl.position = mk( x, y );
	bl.radius = radius;
	bl.falloff = falloff;
	bl.impulsePerLength = impulsePerLength;
	bl.mask = mask;
	int* byRank = hit + w.shapeCap;
	cudaMemsetAsync( byRank, 0xff, sizeof( int ) * (size_t)w.shapeCap, st );
	k_explode_mark<<<grid_for( w.shapeCount ), 256, 0, st>>>( w, bl, hit, byRank );
	if ( w.isl )
		launch_isl_wake_marked( w, st, byRank, w.shapeCap );
	k_explode_apply<<<grid_for( w.bodyCount ), 128, 0, st>>>( w, bl, hit );
}

// b2Shape_TestPoint (shape.c:979-1001, geometry.c:456-502): the point in the
// body frame against the circle, the capsule's segment or, by GJK distance
// without radii, the polygon's core within its radius
__global__ void k_shape_test_point( DWorld w, int s, fv2 point, int* out )
{
	int type = shape_type( w.sflags[s] );
	fxf xf = body_xform( w, w.shapeBody[s] );
	fv2 lp = rinvrot( xf.q, vsub( point, xf.p ) );
	const float4* g = w.geom + (size_t)s * GEOM_F4;
	float4 g0 = g[0], g1 = g[1];
	int r = 0;
	if ( type == ST_CIRCLE )
		r = vdist2( lp, mk( g0.x, g0.y ) ) <= g1.x * g1.x;
	else if ( type == ST_CAPSULE )
	{
		float rr = g1.x * g1.x;
		fv2 p1 = mk( g0.x, g0.y ), p2 = mk( g0.z, g0.w );
		fv2 d = vsub( p2, p1 );
		float dd = vdot( d, d );
		if ( dd == 0.0f )
			r = vdist2( lp, p1 ) <= rr;
		else
		{
			float t = fclamp_s( vdot( vsub( lp, p1 ), d ) / dd, 0.0f, 1.0f );
			r = vdist2( lp, vmuladd( p1, t, d ) ) <= rr;
		}
	}
	else if ( type == ST_POLYGON )
	{
		DProxy pa = blast_proxy( g, ST_POLYGON );
		pa.radius = 0.0f;
		DProxy pb;
		pb.p[0] = lp;
		pb.count = 1;
		pb.radius = 0.0f;
		fxf identity;
		identity.p = mk( 0.0f, 0.0f );
		identity.q.c = 1.0f;
		identity.q.s = 0.0f;
		DCache cache;
		cache.count = 0;
		fv2 pA, pB, n;
		r = gjk_distance( pa, pb, identity, identity, cache, &pA, &pB, &n ) <= g1.x;
	}
	*out = r;
}

void launch_shape_test_point( DWorld& w, cudaStream_t st, int shape, float x, float y, int* out )
{
	k_shape_test_point<<<1, 1, 0, st>>>( w, shape, mk( x, y ), out );
}
