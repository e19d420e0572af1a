// World queries: closest ray hit and AABB overlap.
//
// Box2D v3.1.1 walks its three dynamic trees for these (world.c:2071-2098
// b2World_OverlapAABB tests tree boxes, i.e. fat AABBs, plus
// b2ShouldQueryCollide; world.c:2222-2300 b2World_CastRayClosest clips the
// ray with each hit, ignoring hits at fraction 0). A query here is one thread
// per shape over the device rows: every candidate is tested against the full
// ray and the closest hit is picked with one 64-bit atomicMin on
// (fraction bits, shape id), so ties resolve to the lower shape id.
// Shape ray casts follow geometry.c:506-888 (circle, capsule, segment,
// polygon; a rounded polygon by the shape cast of distance.c:608-697).
#include "dmath.cuh"
#include "dtoi.cuh"
#include "dworld.cuh"
#include "kernels.cuh"

#include "../../include/forge2d_gb300.h"

#include <algorithm>
#include <atomic>
#include <vector>

struct RayHit
{
	bool hit;
	fv2 point, normal;
	float fraction;
};

__device__ RayHit ray_circle( fv2 origin, fv2 translation, float maxFraction, fv2 p, float r )
{
	RayHit out;
	out.hit = false;
	out.fraction = 0.0f;
	out.point = out.normal = mk( 0.0f, 0.0f );
	fv2 s = vsub( origin, p );
	float rr = r * r;
	float length;
	fv2 d = vlen_norm( &length, translation );
	if ( length == 0.0f )
	{
		if ( vlen2( s ) < rr )
		{
			out.point = origin;
			out.hit = true;
		}
		return out;
	}
	float t = -vdot( s, d );
	fv2 c = vmuladd( s, t, d );
	float cc = vdot( c, c );
	if ( cc > rr )
		return out;
	float h = sqrtf( rr - cc );
	float fraction = t - h;
	if ( fraction < 0.0f || maxFraction * length < fraction )
	{
		if ( vlen2( s ) < rr )
		{
			out.point = origin;
			out.hit = true;
		}
		return out;
	}
	fv2 hitPoint = vmuladd( s, fraction, d );
	out.fraction = fraction / length;
	out.normal = vnormalize( hitPoint );
	out.point = vmuladd( p, r, out.normal );
	out.hit = true;
	return out;
}

__device__ RayHit ray_capsule( fv2 origin, fv2 translation, float maxFraction, fv2 v1, fv2 v2, float radius )
{
	RayHit out;
	out.hit = false;
	out.fraction = 0.0f;
	out.point = out.normal = mk( 0.0f, 0.0f );
	fv2 e = vsub( v2, v1 );
	float capsuleLength;
	fv2 a = vlen_norm( &capsuleLength, e );
	if ( capsuleLength < FLT_EPSILON )
		return ray_circle( origin, translation, maxFraction, v1, radius );
	fv2 p1 = origin;
	fv2 d = translation;
	fv2 q = vsub( p1, v1 );
	float qa = vdot( q, a );
	fv2 qp = vmuladd( q, -qa, a );
	if ( vdot( qp, qp ) < radius * radius )
	{
		if ( qa < 0.0f )
			return ray_circle( origin, translation, maxFraction, v1, radius );
		if ( qa > capsuleLength )
			return ray_circle( origin, translation, maxFraction, v2, radius );
		out.point = origin;
		out.hit = true;
		return out;
	}
	fv2 n = mk( a.y, -a.x );
	float rayLength;
	fv2 u = vlen_norm( &rayLength, d );
	float den = -a.x * u.y + u.x * a.y;
	if ( -FLT_EPSILON < den && den < FLT_EPSILON )
		return out;
	fv2 b1 = vmulsub( q, radius, n );
	fv2 b2 = vmuladd( q, radius, n );
	float invDen = 1.0f / den;
	float s21 = ( a.x * b1.y - b1.x * a.y ) * invDen;
	float s22 = ( a.x * b2.y - b2.x * a.y ) * invDen;
	float s2;
	fv2 b;
	if ( s21 < s22 )
	{
		s2 = s21;
		b = b1;
	}
	else
	{
		s2 = s22;
		b = b2;
		n = vneg( n );
	}
	if ( s2 < 0.0f || maxFraction * rayLength < s2 )
		return out;
	float s1 = ( -b.x * u.y + u.x * b.y ) * invDen;
	if ( s1 < 0.0f )
		return ray_circle( origin, translation, maxFraction, v1, radius );
	if ( capsuleLength < s1 )
		return ray_circle( origin, translation, maxFraction, v2, radius );
	out.fraction = s2 / rayLength;
	out.point = vadd( vlerp( v1, v2, s1 / capsuleLength ), vscale( radius, n ) );
	out.normal = n;
	out.hit = true;
	return out;
}

__device__ RayHit ray_segment( fv2 origin, fv2 translation, float maxFraction, fv2 v1, fv2 v2 )
{
	RayHit out;
	out.hit = false;
	out.fraction = 0.0f;
	out.point = out.normal = mk( 0.0f, 0.0f );
	fv2 e = vsub( v2, v1 );
	float length;
	fv2 eUnit = vlen_norm( &length, e );
	if ( length == 0.0f )
		return out;
	fv2 normal = vright( eUnit );
	float numerator = vdot( normal, vsub( v1, origin ) );
	float denominator = vdot( normal, translation );
	if ( denominator == 0.0f )
		return out;
	float t = numerator / denominator;
	if ( t < 0.0f || maxFraction < t )
		return out;
	fv2 p = vmuladd( origin, t, translation );
	float s = vdot( vsub( p, v1 ), eUnit );
	if ( s < 0.0f || length < s )
		return out;
	if ( numerator > 0.0f )
		normal = vneg( normal );
	out.fraction = t;
	out.point = p;
	out.normal = normal;
	out.hit = true;
	return out;
}

// geometry.c:718-729: a chain segment is one-sided; rays starting on its
// left pass through
__device__ RayHit ray_segment_sided( fv2 origin, fv2 translation, fv2 p1, fv2 p2, bool oneSided )
{
	if ( oneSided && vcross( vsub( origin, p1 ), vsub( p2, p1 ) ) < 0.0f )
	{
		RayHit none;
		none.hit = false;
		none.point = mk( 0.0f, 0.0f );
		none.normal = mk( 0.0f, 0.0f );
		none.fraction = 0.0f;
		return none;
	}
	return ray_segment( origin, translation, 1.0f, p1, p2 );
}

// geometry.c:879-888 + distance.c:608-697 b2ShapeCast: the ray's origin
// advances conservatively on the GJK distance (radii off) to the rounded
// polygon until it is within the radius; an initial overlap reports the
// midpoint of the two closest points at fraction 0
__device__ RayHit ray_rounded_polygon( fv2 origin, fv2 d, float maxFraction, const float4* g )
{
	RayHit out;
	out.hit = false;
	out.fraction = 0.0f;
	out.point = out.normal = mk( 0.0f, 0.0f );
	DProxy pa;
	for ( int i = 0; i < 4; ++i )
	{
		float4 a = g[2 + i];
		pa.p[2 * i] = mk( a.x, a.y );
		pa.p[2 * i + 1] = mk( a.z, a.w );
	}
	pa.count = __float_as_int( g[1].y );
	pa.radius = g[1].x;
	DProxy pb;
	pb.p[0] = origin;
	pb.count = 1;
	pb.radius = 0.0f;
	float target = fmax_s( F2D_LINEAR_SLOP, pa.radius + pb.radius - F2D_LINEAR_SLOP );
	float tolerance = 0.25f * F2D_LINEAR_SLOP;
	DCache cache;
	cache.count = 0;
	fxf xfA;
	xfA.p = mk( 0.0f, 0.0f );
	xfA.q.c = 1.0f;
	xfA.q.s = 0.0f;
	fxf xfB = xfA;
	float fraction = 0.0f;
	for ( int iteration = 0; iteration < 20; ++iteration )
	{
		fv2 pA = mk( 0.0f, 0.0f ), pB = mk( 0.0f, 0.0f ), n = mk( 0.0f, 0.0f );
		float dist = gjk_distance( pa, pb, xfA, xfB, cache, &pA, &pB, &n );
		if ( dist < target + tolerance )
		{
			out.hit = true;
			if ( iteration == 0 )
			{
				out.point = vlerp( vmuladd( pA, pa.radius, n ), vmuladd( pB, -pb.radius, n ), 0.5f );
				return out;
			}
			out.fraction = fraction;
			out.point = vmuladd( pA, pa.radius, n );
			out.normal = n;
			return out;
		}
		float den = vdot( d, n );
		if ( den >= 0.0f )
			return out;
		fraction += ( target - dist ) / den;
		if ( fraction >= maxFraction )
			return out;
		xfB.p = vmuladd( mk( 0.0f, 0.0f ), fraction, d );
	}
	return out;
}

__device__ RayHit ray_polygon( fv2 origin, fv2 d, float maxFraction, const float4* g )
{
	if ( g[1].x != 0.0f )
		return ray_rounded_polygon( origin, d, maxFraction, g );
	RayHit out;
	out.hit = false;
	out.fraction = 0.0f;
	out.point = out.normal = mk( 0.0f, 0.0f );
	int count = __float_as_int( g[1].y );
	fv2 v[F2D_MAX_POLY], n[F2D_MAX_POLY];
	for ( int i = 0; i < 4; ++i )
	{
		float4 a = g[2 + i], b = g[6 + i];
		v[2 * i] = mk( a.x, a.y );
		v[2 * i + 1] = mk( a.z, a.w );
		n[2 * i] = mk( b.x, b.y );
		n[2 * i + 1] = mk( b.z, b.w );
	}
	fv2 base = v[0];
	fv2 p1 = vsub( origin, base );
	float lower = 0.0f, upper = maxFraction;
	int index = -1;
	for ( int i = 0; i < count; ++i )
	{
		fv2 vertex = vsub( v[i], base );
		float numerator = vdot( n[i], vsub( vertex, p1 ) );
		float denominator = vdot( n[i], d );
		if ( denominator == 0.0f )
		{
			if ( numerator < 0.0f )
				return out;
		}
		else
		{
			if ( denominator < 0.0f && numerator < lower * denominator )
			{
				lower = numerator / denominator;
				index = i;
			}
			else if ( denominator > 0.0f && numerator < upper * denominator )
				upper = numerator / denominator;
		}
		if ( upper < lower )
			return out;
	}
	if ( index >= 0 )
	{
		out.fraction = lower;
		out.normal = n[index];
		out.point = vmuladd( origin, lower, d );
		out.hit = true;
	}
	else
	{
		out.point = origin;
		out.hit = true;
	}
	return out;
}

__device__ __forceinline__ bool query_collide( const DWorld& w, int s, unsigned long long cat,
											   unsigned long long msk )
{
	return ( w.cat[s] & msk ) != 0ull && ( w.mask[s] & cat ) != 0ull;
}

__device__ __forceinline__ float ray_box_enter( fbox b, fv2 o, fv2 t )
{
	// slab test of the ray segment o + s t, s in [0,1]; returns entry or 2 (miss)
	float tmin = 0.0f, tmax = 1.0f;
	float lo[2] = { b.lo.x, b.lo.y }, hi[2] = { b.hi.x, b.hi.y }, oo[2] = { o.x, o.y }, tt[2] = { t.x, t.y };
	for ( int k = 0; k < 2; ++k )
	{
		if ( fabsf( tt[k] ) < FLT_EPSILON )
		{
			if ( oo[k] < lo[k] || hi[k] < oo[k] )
				return 2.0f;
		}
		else
		{
			float inv = 1.0f / tt[k];
			float t1 = ( lo[k] - oo[k] ) * inv, t2 = ( hi[k] - oo[k] ) * inv;
			if ( t1 > t2 )
			{
				float x = t1;
				t1 = t2;
				t2 = x;
			}
			tmin = fmaxf( tmin, t1 );
			tmax = fminf( tmax, t2 );
			if ( tmin > tmax )
				return 2.0f;
		}
	}
	return tmin;
}

__global__ void k_ray_closest( DWorld w, fv2 origin, fv2 translation, unsigned long long cat, unsigned long long msk,
							   unsigned long long* best )
{
	for ( int s = blockIdx.x * blockDim.x + threadIdx.x; s < w.shapeCount; s += gridDim.x * blockDim.x )
	{
		int f = w.sflags[s];
		if ( ( f & ( SF_USED | SF_PROXY ) ) != ( SF_USED | SF_PROXY ) )
			continue;
		if ( ( w.cat[s] & msk ) == 0ull || !query_collide( w, s, cat, msk ) )
			continue;
		if ( ray_box_enter( box_from4( w.fat[s] ), origin, translation ) > 1.0f )
			continue;
		int b = w.shapeBody[s];
		float4 x4 = w.xf[b];
		fxf xf;
		xf.p = mk( x4.x, x4.y );
		xf.q.c = x4.z;
		xf.q.s = x4.w;
		// shape.c:792-832: cast in the shape's local frame
		fv2 lo = rinvrot( xf.q, vsub( origin, xf.p ) );
		fv2 lt = rinvrot( xf.q, translation );
		const float4* g = w.geom + (size_t)s * GEOM_F4;
		float4 g0 = g[0], g1 = g[1];
		int type = shape_type( f );
		RayHit h;
		if ( type == ST_CIRCLE )
			h = ray_circle( lo, lt, 1.0f, mk( g0.x, g0.y ), g1.x );
		else if ( type == ST_CAPSULE )
			h = ray_capsule( lo, lt, 1.0f, mk( g0.x, g0.y ), mk( g0.z, g0.w ), g1.x );
		else if ( type == ST_SEGMENT || type == ST_CHAIN )
			h = ray_segment_sided( lo, lt, mk( g0.x, g0.y ), mk( g0.z, g0.w ), type == ST_CHAIN );
		else
			h = ray_polygon( lo, lt, 1.0f, g );
		if ( !h.hit || h.fraction == 0.0f )
			continue;
		unsigned long long key = ( (unsigned long long)__float_as_uint( h.fraction ) << 32 ) | (unsigned)s;
		atomicMin( best, key );
	}
}

__global__ void k_ray_result( DWorld w, fv2 origin, fv2 translation, const unsigned long long* best, float* out )
{
	unsigned long long key = *best;
	if ( key == ~0ull )
	{
		out[5] = -1.0f;
		return;
	}
	int s = (int)( key & 0xffffffffull );
	int b = w.shapeBody[s];
	float4 x4 = w.xf[b];
	fxf xf;
	xf.p = mk( x4.x, x4.y );
	xf.q.c = x4.z;
	xf.q.s = x4.w;
	fv2 lo = rinvrot( xf.q, vsub( origin, xf.p ) );
	fv2 lt = rinvrot( xf.q, translation );
	const float4* g = w.geom + (size_t)s * GEOM_F4;
	float4 g0 = g[0], g1 = g[1];
	int type = shape_type( w.sflags[s] );
	RayHit h;
	if ( type == ST_CIRCLE )
		h = ray_circle( lo, lt, 1.0f, mk( g0.x, g0.y ), g1.x );
	else if ( type == ST_CAPSULE )
		h = ray_capsule( lo, lt, 1.0f, mk( g0.x, g0.y ), mk( g0.z, g0.w ), g1.x );
	else if ( type == ST_SEGMENT || type == ST_CHAIN )
		h = ray_segment_sided( lo, lt, mk( g0.x, g0.y ), mk( g0.z, g0.w ), type == ST_CHAIN );
	else
		h = ray_polygon( lo, lt, 1.0f, g );
	fv2 p = xpoint( xf, h.point );
	fv2 n = rrot( xf.q, h.normal );
	out[0] = p.x;
	out[1] = p.y;
	out[2] = n.x;
	out[3] = n.y;
	out[4] = h.fraction;
	out[5] = __int_as_float( s );
}

__global__ void k_overlap( DWorld w, fbox box, unsigned long long cat, unsigned long long msk, int* out, int* count,
						   int cap )
{
	for ( int s = blockIdx.x * blockDim.x + threadIdx.x; s < w.shapeCount; s += gridDim.x * blockDim.x )
	{
		int f = w.sflags[s];
		if ( ( f & ( SF_USED | SF_PROXY ) ) != ( SF_USED | SF_PROXY ) )
			continue;
		if ( ( w.cat[s] & msk ) == 0ull || !query_collide( w, s, cat, msk ) )
			continue;
		if ( !box_overlaps( box_from4( w.fat[s] ), box ) )
			continue;
		int k = atomicAdd( count, 1 );
		if ( k < cap )
			out[k] = s;
	}
}

// ---------------------------------------------------------------------------
// host entry points (world.cu owns the world table)
// ---------------------------------------------------------------------------
DWorld* f2d_internal_world( int32_t worldId, cudaStream_t* st, int* gens, int genCap );
uint16_t f2d_internal_shape_gen( int32_t worldId, int shape );
int32_t f2d_internal_world0( int32_t worldId );

extern "C" F2D_API int32_t f2d_world_cast_ray_closest( int32_t worldId, double ox, double oy, double tx, double ty,
													   int64_t categoryBits, int64_t maskBits, int32_t* shape2,
													   float* out5 )
{
	cudaStream_t st;
	DWorld* w = f2d_internal_world( worldId, &st, nullptr, 0 );
	if ( w == nullptr )
		return 0;
	unsigned long long* best = nullptr;
	float* res = nullptr;
	cudaMalloc( (void**)&best, sizeof( unsigned long long ) );
	cudaMalloc( (void**)&res, 6 * sizeof( float ) );
	cudaMemsetAsync( best, 0xff, sizeof( unsigned long long ), st );
	fv2 o = mk( (float)ox, (float)oy ), t = mk( (float)tx, (float)ty );
	k_ray_closest<<<grid_for( w->shapeCount ), 256, 0, st>>>( *w, o, t, (unsigned long long)categoryBits,
															   (unsigned long long)maskBits, best );
	k_ray_result<<<1, 1, 0, st>>>( *w, o, t, best, res );
	float h[6];
	cudaMemcpyAsync( h, res, sizeof( h ), cudaMemcpyDeviceToHost, st );
	cudaStreamSynchronize( st );
	cudaFree( best );
	cudaFree( res );
	if ( h[5] == -1.0f )
		return 0;
	int s;
	memcpy( &s, &h[5], sizeof( int ) );
	if ( shape2 )
	{
		shape2[0] = s + 1;
		shape2[1] = f2d_internal_world0( worldId ) | ( (int)f2d_internal_shape_gen( worldId, s ) << 16 );
	}
	if ( out5 )
		for ( int k = 0; k < 5; ++k )
			out5[k] = h[k];
	return 1;
}

// Every hit of the whole ray (callback form of b2World_CastRay): shape id
// and point, normal, fraction in the world frame
__global__ void k_ray_all( DWorld w, fv2 origin, fv2 translation, unsigned long long cat, unsigned long long msk,
						   int* count, int* shapes, float* rows )
{
	for ( int s = blockIdx.x * blockDim.x + threadIdx.x; s < w.shapeCount; s += gridDim.x * blockDim.x )
	{
		int f = w.sflags[s];
		if ( ( f & ( SF_USED | SF_PROXY ) ) != ( SF_USED | SF_PROXY ) )
			continue;
		if ( ( w.cat[s] & msk ) == 0ull || !query_collide( w, s, cat, msk ) )
			continue;
		if ( ray_box_enter( box_from4( w.fat[s] ), origin, translation ) > 1.0f )
			continue;
		int b = w.shapeBody[s];
		float4 x4 = w.xf[b];
		fxf xf;
		xf.p = mk( x4.x, x4.y );
		xf.q.c = x4.z;
		xf.q.s = x4.w;
		fv2 lo = rinvrot( xf.q, vsub( origin, xf.p ) );
		fv2 lt = rinvrot( xf.q, translation );
		const float4* g = w.geom + (size_t)s * GEOM_F4;
		float4 g0 = g[0], g1 = g[1];
		int type = shape_type( f );
		RayHit h;
		if ( type == ST_CIRCLE )
			h = ray_circle( lo, lt, 1.0f, mk( g0.x, g0.y ), g1.x );
		else if ( type == ST_CAPSULE )
			h = ray_capsule( lo, lt, 1.0f, mk( g0.x, g0.y ), mk( g0.z, g0.w ), g1.x );
		else if ( type == ST_SEGMENT || type == ST_CHAIN )
			h = ray_segment_sided( lo, lt, mk( g0.x, g0.y ), mk( g0.z, g0.w ), type == ST_CHAIN );
		else
			h = ray_polygon( lo, lt, 1.0f, g );
		if ( !h.hit )
			continue;
		int slot = atomicAdd( count, 1 );
		fv2 p = xpoint( xf, h.point );
		fv2 n = rrot( xf.q, h.normal );
		shapes[slot] = s;
		float* r = rows + 5 * (size_t)slot;
		r[0] = p.x;
		r[1] = p.y;
		r[2] = n.x;
		r[3] = n.y;
		r[4] = h.fraction;
	}
}

// RawBox2D.worldCastRay (raw_box2d.dart:1318 -> b2World_CastRay, world.c:
// 2176-2251): the callback sees the ray's hits in ascending fraction (then
// shape id), the order in which a ray clipped by every returned fraction
// meets them; a hit past the current clip is not reported, 0 ends the cast,
// -1 skips the hit, a fraction in [0, 1] clips. Returns the number of calls.
extern "C" F2D_API int32_t f2d_world_cast_ray( int32_t worldId, double ox, double oy, double tx, double ty,
											   int64_t categoryBits, int64_t maskBits, f2d_cast_result_fn fn,
											   void* context )
{
	cudaStream_t st;
	DWorld* w = f2d_internal_world( worldId, &st, nullptr, 0 );
	if ( w == nullptr || fn == nullptr || w->shapeCount == 0 )
		return 0;
	int n = w->shapeCount;
	int* dCount = nullptr;
	int* dShapes = nullptr;
	float* dRows = nullptr;
	cudaMalloc( (void**)&dCount, sizeof( int ) );
	cudaMalloc( (void**)&dShapes, sizeof( int ) * (size_t)n );
	cudaMalloc( (void**)&dRows, sizeof( float ) * 5 * (size_t)n );
	cudaMemsetAsync( dCount, 0, sizeof( int ), st );
	fv2 o = mk( (float)ox, (float)oy ), t = mk( (float)tx, (float)ty );
	k_ray_all<<<grid_for( n ), 256, 0, st>>>( *w, o, t, (unsigned long long)categoryBits, (unsigned long long)maskBits,
											  dCount, dShapes, dRows );
	int m = 0;
	cudaMemcpyAsync( &m, dCount, sizeof( int ), cudaMemcpyDeviceToHost, st );
	cudaStreamSynchronize( st );
	m = std::min( m, n );
	std::vector<int> shapes( (size_t)m );
	std::vector<float> rows( 5 * (size_t)m );
	if ( m > 0 )
	{
		cudaMemcpy( shapes.data(), dShapes, sizeof( int ) * m, cudaMemcpyDeviceToHost );
		cudaMemcpy( rows.data(), dRows, sizeof( float ) * 5 * m, cudaMemcpyDeviceToHost );
	}
	cudaFree( dCount );
	cudaFree( dShapes );
	cudaFree( dRows );
	std::vector<int> order( (size_t)m );
	for ( int i = 0; i < m; ++i )
		order[i] = i;
	std::sort( order.begin(), order.end(), [&]( int a, int b ) {
		float fa = rows[5 * (size_t)a + 4], fb = rows[5 * (size_t)b + 4];
		return fa != fb ? fa < fb : shapes[a] < shapes[b];
	} );
	float clip = 1.0f;
	int calls = 0;
	int world0 = f2d_internal_world0( worldId );
	for ( int k : order )
	{
		const float* r = rows.data() + 5 * (size_t)k;
		if ( r[4] > clip )
			break;
		int s = shapes[k];
		float v = fn( s + 1, world0 | ( (int)f2d_internal_shape_gen( worldId, s ) << 16 ), r[0], r[1], r[2], r[3], r[4],
					  context );
		calls += 1;
		if ( v == 0.0f )
			break;
		if ( 0.0f <= v && v <= 1.0f )
			clip = v;
	}
	return calls;
}

extern "C" F2D_API int32_t f2d_world_overlap_aabb( int32_t worldId, double lx, double ly, double ux, double uy,
												   int64_t categoryBits, int64_t maskBits, int32_t* shapes2,
												   int32_t capacity )
{
	cudaStream_t st;
	DWorld* w = f2d_internal_world( worldId, &st, nullptr, 0 );
	if ( w == nullptr )
		return 0;
	int cap = w->shapeCount > 0 ? w->shapeCount : 1;
	int* out = nullptr;
	int* count = nullptr;
	cudaMalloc( (void**)&out, sizeof( int ) * cap );
	cudaMalloc( (void**)&count, sizeof( int ) );
	cudaMemsetAsync( count, 0, sizeof( int ), st );
	fbox box;
	box.lo = mk( (float)lx, (float)ly );
	box.hi = mk( (float)ux, (float)uy );
	k_overlap<<<grid_for( w->shapeCount ), 256, 0, st>>>( *w, box, (unsigned long long)categoryBits,
														   (unsigned long long)maskBits, out, count, cap );
	int n = 0;
	cudaMemcpyAsync( &n, count, sizeof( int ), cudaMemcpyDeviceToHost, st );
	cudaStreamSynchronize( st );
	std::vector<int> ids( std::min( n, cap ) );
	if ( !ids.empty() )
		cudaMemcpy( ids.data(), out, sizeof( int ) * ids.size(), cudaMemcpyDeviceToHost );
	cudaFree( out );
	cudaFree( count );
	std::sort( ids.begin(), ids.end() );
	int world0 = f2d_internal_world0( worldId );
	for ( int i = 0; i < (int)ids.size() && i < capacity; ++i )
	{
		shapes2[2 * i] = ids[i] + 1;
		shapes2[2 * i + 1] = world0 | ( (int)f2d_internal_shape_gen( worldId, ids[i] ) << 16 );
	}
	return n;
}

// ---------------------------------------------------------------------------
// Allocation-free AABB overlap. The scratch is one file-scope device array:
// per-block hit counts, their exclusive scan and the compacted shape ids.
// Three launches make the result order ascending by construction (count per
// block, scan the counts, write each hit at its block's base plus its rank in
// the block), so no sort and no host buffer is needed.
// ---------------------------------------------------------------------------
#define OVERLAP_BLOCK 256
#define OVERLAP_NOALLOC_BLOCKS ( F2D_OVERLAP_NOALLOC_MAX_SHAPES / OVERLAP_BLOCK )
#define NOALLOC_MAX_DEVICES 64

static_assert( OVERLAP_NOALLOC_BLOCKS <= 1024, "the scan kernel runs one 1024-thread block" );

struct OverlapScratch
{
	int total;
	int pad[63];
	int blockBase[OVERLAP_NOALLOC_BLOCKS];
	int ids[F2D_OVERLAP_NOALLOC_MAX_SHAPES];
};

static __device__ __align__( 256 ) OverlapScratch g_overlapScratch;

// device address of g_overlapScratch per device ordinal, resolved on first
// use; host threads may race to resolve it, so the cache entries are atomic
// (every thread stores the same address)
static std::atomic<OverlapScratch*> s_overlapScratch[NOALLOC_MAX_DEVICES];

static OverlapScratch* overlap_scratch()
{
	int dev = 0;
	if ( cudaGetDevice( &dev ) != cudaSuccess || dev < 0 || dev >= NOALLOC_MAX_DEVICES )
		return nullptr;
	OverlapScratch* cached = s_overlapScratch[dev].load( std::memory_order_acquire );
	if ( cached == nullptr )
	{
		void* p = nullptr;
		if ( cudaGetSymbolAddress( &p, g_overlapScratch ) != cudaSuccess )
			return nullptr;
		cached = (OverlapScratch*)p;
		s_overlapScratch[dev].store( cached, std::memory_order_release );
	}
	return cached;
}

__device__ __forceinline__ bool overlap_hit( const DWorld& w, int s, fbox box, unsigned long long cat,
											 unsigned long long msk )
{
	if ( s >= w.shapeCount )
		return false;
	int f = w.sflags[s];
	if ( ( f & ( SF_USED | SF_PROXY ) ) != ( SF_USED | SF_PROXY ) )
		return false;
	if ( !query_collide( w, s, cat, msk ) )
		return false;
	return box_overlaps( box_from4( w.fat[s] ), box );
}

__global__ void __launch_bounds__( OVERLAP_BLOCK ) k_overlap_count( DWorld w, fbox box, unsigned long long cat,
																	 unsigned long long msk, OverlapScratch* scr )
{
	int s = blockIdx.x * OVERLAP_BLOCK + threadIdx.x;
	int c = __syncthreads_count( overlap_hit( w, s, box, cat, msk ) );
	if ( threadIdx.x == 0 )
		scr->blockBase[blockIdx.x] = c;
}

// exclusive scan of the per-block counts; one block of 1024 threads
__global__ void __launch_bounds__( 1024 ) k_overlap_scan( OverlapScratch* scr, int blocks )
{
	__shared__ int warpSum[32];
	int t = threadIdx.x, lane = t & 31, wid = t >> 5;
	int v = t < blocks ? scr->blockBase[t] : 0;
	int x = v;
	for ( int o = 1; o < 32; o <<= 1 )
	{
		int y = __shfl_up_sync( 0xffffffffu, x, o );
		if ( lane >= o )
			x += y;
	}
	if ( lane == 31 )
		warpSum[wid] = x;
	__syncthreads();
	if ( wid == 0 )
	{
		int ws = warpSum[lane];
		for ( int o = 1; o < 32; o <<= 1 )
		{
			int y = __shfl_up_sync( 0xffffffffu, ws, o );
			if ( lane >= o )
				ws += y;
		}
		warpSum[lane] = ws;
	}
	__syncthreads();
	int inclusive = x + ( wid > 0 ? warpSum[wid - 1] : 0 );
	if ( t < blocks )
		scr->blockBase[t] = inclusive - v;
	if ( t == 1023 )
		scr->total = inclusive;
}

__global__ void __launch_bounds__( OVERLAP_BLOCK ) k_overlap_write( DWorld w, fbox box, unsigned long long cat,
																	 unsigned long long msk, OverlapScratch* scr )
{
	__shared__ int warpBase[OVERLAP_BLOCK / 32];
	int s = blockIdx.x * OVERLAP_BLOCK + threadIdx.x;
	int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
	bool hit = overlap_hit( w, s, box, cat, msk );
	unsigned ballot = __ballot_sync( 0xffffffffu, hit );
	if ( lane == 0 )
		warpBase[wid] = __popc( ballot );
	__syncthreads();
	if ( threadIdx.x == 0 )
	{
		int acc = 0;
		for ( int k = 0; k < OVERLAP_BLOCK / 32; ++k )
		{
			int c = warpBase[k];
			warpBase[k] = acc;
			acc += c;
		}
	}
	__syncthreads();
	if ( hit )
		scr->ids[scr->blockBase[blockIdx.x] + warpBase[wid] + __popc( ballot & ( ( 1u << lane ) - 1u ) )] = s;
}

DWorld* f2d_internal_world_noalloc( int32_t worldId, cudaStream_t* st, int maxShapes, int* code );

extern "C" F2D_API int32_t f2d_world_overlap_aabb_noalloc( int32_t worldId, double lx, double ly, double ux,
														   double uy, int64_t categoryBits, int64_t maskBits,
														   int32_t* shapes2, int32_t capacity )
{
	cudaStream_t st;
	int code = 0;
	DWorld* w = f2d_internal_world_noalloc( worldId, &st, F2D_OVERLAP_NOALLOC_MAX_SHAPES, &code );
	if ( w == nullptr )
		return code;
	OverlapScratch* scr = overlap_scratch();
	if ( scr == nullptr )
		return F2D_NOALLOC_DEVICE_SETUP;
	int shapeCount = w->shapeCount;
	if ( shapeCount == 0 )
		return 0;
	int blocks = ( shapeCount + OVERLAP_BLOCK - 1 ) / OVERLAP_BLOCK;
	fbox box;
	box.lo = mk( (float)lx, (float)ly );
	box.hi = mk( (float)ux, (float)uy );
	unsigned long long cat = (unsigned long long)categoryBits, msk = (unsigned long long)maskBits;
	k_overlap_count<<<blocks, OVERLAP_BLOCK, 0, st>>>( *w, box, cat, msk, scr );
	k_overlap_scan<<<1, 1024, 0, st>>>( scr, blocks );
	k_overlap_write<<<blocks, OVERLAP_BLOCK, 0, st>>>( *w, box, cat, msk, scr );
	int n = 0;
	cudaMemcpyAsync( &n, &scr->total, sizeof( int ), cudaMemcpyDeviceToHost, st );
	cudaStreamSynchronize( st );
	int m = n < capacity ? n : capacity;
	if ( m <= 0 || shapes2 == nullptr )
		return n;
	cudaMemcpyAsync( shapes2, scr->ids, sizeof( int ) * (size_t)m, cudaMemcpyDeviceToHost, st );
	cudaStreamSynchronize( st );
	// widen shape indices to (index1, worldAndGeneration) pairs in place, back to front
	int world0 = f2d_internal_world0( worldId );
	for ( int i = m - 1; i >= 0; --i )
	{
		int s = shapes2[i];
		shapes2[2 * i + 1] = world0 | ( (int)f2d_internal_shape_gen( worldId, s ) << 16 );
		shapes2[2 * i] = s + 1;
	}
	return n;
}
