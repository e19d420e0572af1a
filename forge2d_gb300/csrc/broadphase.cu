// Broadphase of the world step: the new contact pairs, in the reference's
// creation order.
//
// Box2D v3.1.1 keeps three incremental dynamic trees and queries them with
// every moved proxy (broad_phase.c:160-474, dynamic_tree.c:1114). The pair
// SET that produces is: every pair of shapes with overlapping fat AABBs, at
// least one of them a dynamic proxy and at least one of them moved, that
// passes the filters and has no contact yet. This file finds that set
// GPU-first:
//   1. an implicit 32-ary bounding-volume tree over all proxies' fat AABBs:
//      leaves in the order of their 30-bit Morton codes (one-launch radix
//      sort), node k of level l bounding children 32k..32k+31 of level l-1,
//      so no topology is stored and a refit is one launch whose longest
//      dependency chain is the tree height (4 levels at 1e6 proxies);
//   2. one warp per moved proxy walks it depth first, the 32 children of a
//      node tested by the 32 lanes at once;
//   3. each pair is kept by the proxy whose query creates it in the
//      reference, with the key (that proxy's move-array position, tree of
//      the other proxy, the other proxy's left-to-right rank in the
//      reference's tree, found by a walk to the root) and the other shape as
//      the sorted value; the reference's trees are kept in proxytree.cu.
//      Sorting the keys gives the reference's creation order, in which
//      contact ids are then drawn from the LIFO id pool.
#include "dscan.cuh"
#include "dsort.cuh"
#include "dtree.cuh"
#include "dworld.cuh"
#include "kernels.cuh"

#define BP_THREADS 256
// refit counters exist for the nodes of levels >= 2
__device__ __forceinline__ int wide_counter( const WideLevels& L, int level, int node )
{
	return L.offset[level] - L.offset[2] + node;
}

__device__ __forceinline__ unsigned long long pair_key( int a, int b )
{
	return a < b ? ( ( (unsigned long long)a << 32 ) | (unsigned)b ) : ( ( (unsigned long long)b << 32 ) | (unsigned)a );
}

__device__ __forceinline__ unsigned hash64( unsigned long long k )
{
	k ^= k >> 33;
	k *= 0xff51afd7ed558ccdULL;
	k ^= k >> 33;
	k *= 0xc4ceb9fe1a85ec53ULL;
	k ^= k >> 33;
	return (unsigned)k;
}

// ---------------------------------------------------------------------------
// pair set: rebuilt every step from the live contacts (no deletions needed)
// ---------------------------------------------------------------------------
__global__ void k_hash_clear( DWorld w )
{
	for ( int i = blockIdx.x * blockDim.x + threadIdx.x; i < w.hashCap; i += gridDim.x * blockDim.x )
		w.pairHash[i] = 0ull;
	// refit counters of the implicit tree (levels >= 2 hold fewer than one
	// node per 1000 leaves), used by k_wide_refit
	int counters = min( w.shapeCap, w.shapeCount / 512 + 8 );
	for ( int i = blockIdx.x * blockDim.x + threadIdx.x; i < counters; i += gridDim.x * blockDim.x )
		w.nodeVisit[i] = 0;
}

__global__ void k_hash_insert( DWorld w )
{
	int n = w.sc->contactIdCount;
	unsigned m = (unsigned)w.hashCap - 1u;
	for ( int c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x )
	{
		if ( ( w.cflags[c] & CF_USED ) == 0 )
			continue;
		int2 s = w.cshape[c];
		unsigned long long key = pair_key( s.x, s.y ) + 1ull;
		unsigned h = hash64( key - 1ull ) & m;
		for ( int probe = 0; probe < w.hashCap; ++probe )
		{
			unsigned long long prev = atomicCAS( w.pairHash + h, 0ull, key );
			if ( prev == 0ull || prev == key )
				break;
			h = ( h + 1u ) & m;
		}
	}
}

__device__ __forceinline__ bool hash_contains( const DWorld& w, unsigned long long key )
{
	unsigned m = (unsigned)w.hashCap - 1u;
	unsigned h = hash64( key ) & m;
	unsigned long long k1 = key + 1ull;
	for ( int probe = 0; probe < w.hashCap; ++probe )
	{
		unsigned long long v = w.pairHash[h];
		if ( v == 0ull )
			return false;
		if ( v == k1 )
			return true;
		h = ( h + 1u ) & m;
	}
	return false;
}

// ---------------------------------------------------------------------------
// LBVH build
// ---------------------------------------------------------------------------
__global__ void k_leaf_flags( DWorld w, int* flags )
{
	if ( w.sc->rebuildOrder == 0 )
		return;
	for ( int s = blockIdx.x * blockDim.x + threadIdx.x; s < w.shapeCount; s += gridDim.x * blockDim.x )
		flags[s] = ( w.sflags[s] & ( SF_USED | SF_PROXY ) ) == ( SF_USED | SF_PROXY ) ? 1 : 0;
}

__global__ void k_leaf_compact( DWorld w, const int* flags, const int* offs )
{
	if ( w.sc->rebuildOrder == 0 )
		return;
	for ( int s = blockIdx.x * blockDim.x + threadIdx.x; s < w.shapeCount; s += gridDim.x * blockDim.x )
		if ( flags[s] )
			w.leafShape[offs[s]] = s;
}

// block min/max of fat-box centres, then a single-block final reduction
__global__ void k_bounds_partial( DWorld w, float4* partial )
{
	__shared__ float4 red[BP_THREADS];
	if ( w.sc->rebuildOrder == 0 )
		return;
	int n = w.sc->treeLeafCount;
	float4 b = make_float4( FLT_MAX, FLT_MAX, -FLT_MAX, -FLT_MAX );
	for ( int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x )
	{
		float4 f = w.fat[w.leafShape[i]];
		float cx = 0.5f * ( f.x + f.z ), cy = 0.5f * ( f.y + f.w );
		b.x = fminf( b.x, cx );
		b.y = fminf( b.y, cy );
		b.z = fmaxf( b.z, cx );
		b.w = fmaxf( b.w, cy );
	}
	red[threadIdx.x] = b;
	__syncthreads();
	for ( int o = blockDim.x / 2; o > 0; o >>= 1 )
	{
		if ( threadIdx.x < o )
		{
			float4 a = red[threadIdx.x], c = red[threadIdx.x + o];
			red[threadIdx.x] = make_float4( fminf( a.x, c.x ), fminf( a.y, c.y ), fmaxf( a.z, c.z ), fmaxf( a.w, c.w ) );
		}
		__syncthreads();
	}
	if ( threadIdx.x == 0 )
		partial[blockIdx.x] = red[0];
}

__global__ void k_bounds_final( const int* rebuild, float4* partial, int count )
{
	__shared__ float4 red[BP_THREADS];
	if ( *rebuild == 0 )
		return;
	float4 b = make_float4( FLT_MAX, FLT_MAX, -FLT_MAX, -FLT_MAX );
	for ( int i = threadIdx.x; i < count; i += blockDim.x )
	{
		float4 a = partial[i];
		b = make_float4( fminf( a.x, b.x ), fminf( a.y, b.y ), fmaxf( a.z, b.z ), fmaxf( a.w, b.w ) );
	}
	red[threadIdx.x] = b;
	__syncthreads();
	for ( int o = blockDim.x / 2; o > 0; o >>= 1 )
	{
		if ( threadIdx.x < o )
		{
			float4 a = red[threadIdx.x], c = red[threadIdx.x + o];
			red[threadIdx.x] = make_float4( fminf( a.x, c.x ), fminf( a.y, c.y ), fmaxf( a.z, c.z ), fmaxf( a.w, c.w ) );
		}
		__syncthreads();
	}
	if ( threadIdx.x == 0 )
		partial[0] = red[0];
}

__device__ __forceinline__ unsigned expand_bits15( unsigned v )
{
	v &= 0x7fffu;
	v = ( v | ( v << 8 ) ) & 0x00ff00ffu;
	v = ( v | ( v << 4 ) ) & 0x0f0f0f0fu;
	v = ( v | ( v << 2 ) ) & 0x33333333u;
	v = ( v | ( v << 1 ) ) & 0x55555555u;
	return v;
}

__global__ void k_morton( DWorld w, const float4* bounds )
{
	if ( w.sc->rebuildOrder == 0 )
		return;
	int n = w.sc->treeLeafCount;
	float4 b = bounds[0];
	float sx = b.z - b.x, sy = b.w - b.y;
	float inx = sx > 0.0f ? 32767.0f / sx : 0.0f;
	float iny = sy > 0.0f ? 32767.0f / sy : 0.0f;
	for ( int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x )
	{
		float4 f = w.fat[w.leafShape[i]];
		float cx = 0.5f * ( f.x + f.z ), cy = 0.5f * ( f.y + f.w );
		unsigned qx = (unsigned)fminf( fmaxf( ( cx - b.x ) * inx, 0.0f ), 32767.0f );
		unsigned qy = (unsigned)fminf( fmaxf( ( cy - b.y ) * iny, 0.0f ), 32767.0f );
		w.mortonKeys[i] = ( expand_bits15( qx ) << 1 ) | expand_bits15( qy );
	}
}

__device__ __forceinline__ float4 box_union4( float4 a, float4 b )
{
	return make_float4( fminf( a.x, b.x ), fminf( a.y, b.y ), fmaxf( a.z, b.z ), fmaxf( a.w, b.w ) );
}

__device__ __forceinline__ float4 warp_box_union( float4 b )
{
#pragma unroll
	for ( int o = 16; o > 0; o >>= 1 )
	{
		float4 t;
		t.x = __shfl_xor_sync( 0xffffffffu, b.x, o );
		t.y = __shfl_xor_sync( 0xffffffffu, b.y, o );
		t.z = __shfl_xor_sync( 0xffffffffu, b.z, o );
		t.w = __shfl_xor_sync( 0xffffffffu, b.w, o );
		b = box_union4( b, t );
	}
	return b;
}

__device__ __forceinline__ int atom_add_acq_rel( int* p, int v )
{
	int old;
	asm volatile( "atom.acq_rel.gpu.global.add.s32 %0, [%1], %2;" : "=r"( old ) : "l"( p ), "r"( v ) : "memory" );
	return old;
}

// One warp per level-1 node: the 32 leaf boxes (fat AABBs in Morton order)
// and their union. The last child to finish a node of level >= 2 (atomic
// counter) unions that node's children, up to the root.
__global__ void k_wide_refit( DWorld w )
{
	const int n = w.sc->treeLeafCount;
	const WideLevels L = wide_levels( n );
	const int lane = threadIdx.x & 31;
	const int warps = ( gridDim.x * blockDim.x ) >> 5;
	const float4 empty = make_float4( FLT_MAX, FLT_MAX, -FLT_MAX, -FLT_MAX );
	const int groups = ( n + WIDE - 1 ) / WIDE;
	for ( int g = ( blockIdx.x * blockDim.x + threadIdx.x ) >> 5; g < groups; g += warps )
	{
		int i = g * WIDE + lane;
		float4 b = empty;
		if ( i < n )
		{
			b = w.fat[w.leafShape[i]];
			w.nodeBox[i] = b;
		}
		if ( L.top == 0 )
			continue;
		b = warp_box_union( b );
		if ( lane == 0 )
			w.nodeBox[L.offset[1] + g] = b;
		int level = 1, node = g;
		while ( level < L.top )
		{
			int parent = node / WIDE;
			int nchild = min( WIDE, L.count[level] - parent * WIDE );
			int prev = 0;
			if ( lane == 0 )
				prev = atom_add_acq_rel( w.nodeVisit + wide_counter( L, level + 1, parent ), 1 );
			prev = __shfl_sync( 0xffffffffu, prev, 0 );
			if ( prev != nchild - 1 )
				break;
			__threadfence();
			int ci = parent * WIDE + lane;
			float4 cb = lane < nchild ? __ldcg( w.nodeBox + L.offset[level] + ci ) : empty;
			cb = warp_box_union( cb );
			level += 1;
			node = parent;
			if ( lane == 0 )
				w.nodeBox[L.offset[level] + node] = cb;
		}
	}
}

// ---------------------------------------------------------------------------
// pair filters (shape.h:122-130, body.c:1861-1897)
// ---------------------------------------------------------------------------
__device__ __forceinline__ bool shapes_collide( const DWorld& w, int a, int b )
{
	int ga = w.group[a], gb = w.group[b];
	if ( ga == gb && ga != 0 )
		return ga > 0;
	return ( w.mask[a] & w.cat[b] ) != 0ull && ( w.cat[a] & w.mask[b] ) != 0ull;
}

__device__ __forceinline__ bool bodies_collide( const DWorld& w, int ia, int ib )
{
	int fa = w.bflags[ia], fb = w.bflags[ib];
	if ( body_type( fa ) != 2 && body_type( fb ) != 2 )
		return false;
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

__device__ __forceinline__ bool registered( int ta, int tb, bool* primary )
{
	// contact.c:151-184 registry: (first, second) has a manifold function
	// circle-circle, capsule-circle, capsule-capsule, polygon-circle,
	// polygon-capsule, polygon-polygon, segment-circle, segment-capsule,
	// segment-polygon, chain-circle, chain-capsule, chain-polygon
	const unsigned reg = ( 1u << ( 0 * 5 + 0 ) ) | ( 1u << ( 1 * 5 + 0 ) ) | ( 1u << ( 1 * 5 + 1 ) ) |
						 ( 1u << ( 3 * 5 + 0 ) ) | ( 1u << ( 3 * 5 + 1 ) ) | ( 1u << ( 3 * 5 + 3 ) ) |
						 ( 1u << ( 2 * 5 + 0 ) ) | ( 1u << ( 2 * 5 + 1 ) ) | ( 1u << ( 2 * 5 + 3 ) ) |
						 ( 1u << ( 4 * 5 + 0 ) ) | ( 1u << ( 4 * 5 + 1 ) ) | ( 1u << ( 4 * 5 + 3 ) );
	if ( reg & ( 1u << ( ta * 5 + tb ) ) )
	{
		*primary = true;
		return true;
	}
	if ( reg & ( 1u << ( tb * 5 + ta ) ) )
	{
		*primary = false;
		return true;
	}
	*primary = true;
	return false;
}

// Candidate pair (si moved, sj its overlapping leaf): the filters of
// b2PairQueryCallback (broad_phase.c:160-266) and the pair-set lookup. A
// pair whose proxies both moved belongs to one query in the reference: the
// smaller proxy key's when both are dynamic, else the dynamic proxy's (a
// static or kinematic proxy queries the dynamic tree only and skips moved
// proxies there).
__device__ __forceinline__ void test_pair( const DWorld& w, int si, int fi, int typeI, int bi, int sj )
{
	if ( sj == si || ( w.subCount > 0 && w.shapeSub[si] != w.shapeSub[sj] ) )
		return;
	int fj = w.sflags[sj];
	int keyI = w.proxyKey[si], keyJ = w.proxyKey[sj];
	int typeJ = keyJ & 3;
	if ( typeI != 2 && typeJ != 2 )
		return;
	if ( fj & SF_MOVED )
	{
		if ( typeI == 2 && typeJ == 2 ? keyJ < keyI : typeI != 2 )
			return; // created by sj's query
	}
	// dynamic_tree.c:1140: a leaf of category zero is never visited
	if ( w.cat[sj] == 0ull )
		return;
	bool primaryUnused;
	if ( !registered( shape_type( fi ), shape_type( fj ), &primaryUnused ) )
		return; // no manifold function: b2CreateContact makes no contact
	int bj = w.shapeBody[sj];
	if ( bj == bi || ( fi & SF_SENSOR ) || ( fj & SF_SENSOR ) )
		return;
	if ( !shapes_collide( w, si, sj ) || !bodies_collide( w, bi, bj ) )
		return;
	if ( hash_contains( w, pair_key( si, sj ) ) )
		return;
	int slot = atomicAdd( &w.sc->newPairCount, 1 );
	if ( slot < w.pairCap )
	{
		// tree order of a query's pairs after the prepends: dynamic, static,
		// kinematic, each left to right
		int rb = w.pairKeyBits;
		unsigned long long tord = typeJ == 2 ? 0ull : ( typeJ == 0 ? 1ull : 2ull );
		unsigned long long rank = (unsigned)tree_leaf_rank( w.pt[typeJ], keyJ >> 2 );
		w.pairKeys[slot] = ( (unsigned long long)w.shapeMove[si] << ( rb + 2 ) ) | ( tord << rb ) | rank;
		w.pairVal[slot] = sj;
	}
	else
		atomicOr( &w.sc->error, ERR_PAIR_CAPACITY );
}

// One warp per moved proxy: the 32 children of a node are tested by the 32
// lanes at once (one coalesced load), overlapping inner children are pushed
// on a per-warp stack in shared memory, overlapping leaves are tested by
// their lanes in parallel. The visiting order does not matter: new pairs are
// sorted by their keys afterwards.
#define FIND_WARPS ( BP_THREADS / 32 )
#define FIND_STACK ( WIDE * WIDE_MAX_LEVELS )

__global__ void __launch_bounds__( BP_THREADS ) k_find_pairs( DWorld w )
{
	__shared__ int stack[FIND_WARPS][FIND_STACK];
	const int n = w.sc->treeLeafCount;
	if ( n < 2 )
		return;
	const WideLevels L = wide_levels( n );
	const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
	const unsigned below = ( 1u << lane ) - 1u;
	int* stk = stack[wib];
	const int warps = ( gridDim.x * blockDim.x ) >> 5;
	for ( int li = ( blockIdx.x * blockDim.x + threadIdx.x ) >> 5; li < n; li += warps )
	{
		int si = w.leafShape[li];
		int fi = w.sflags[si];
		if ( ( fi & SF_MOVED ) == 0 )
			continue;
		int typeI = w.proxyKey[si] & 3;
		fbox q = box_from4( w.fat[si] );
		int bi = w.shapeBody[si];
		// stack entries: level << 26 | node
		int sp = 1;
		if ( lane == 0 )
			stk[0] = L.top << 26;
		__syncwarp();
		for ( int guard = 0; sp > 0; ++guard )
		{
			if ( guard > 2 * n + 64 )
			{
				if ( lane == 0 )
					atomicOr( &w.sc->error, ERR_TREE );
				break;
			}
			sp -= 1;
			int e = stk[sp];
			__syncwarp();
			int level = e >> 26, node = e & ( ( 1 << 26 ) - 1 );
			int nchild = min( WIDE, L.count[level - 1] - node * WIDE );
			int child = node * WIDE + lane;
			bool ov = lane < nchild && box_overlaps( q, box_from4( w.nodeBox[L.offset[level - 1] + child] ) );
			unsigned mask = __ballot_sync( 0xffffffffu, ov );
			if ( level == 1 )
			{
				if ( ov )
					test_pair( w, si, fi, typeI, bi, w.leafShape[child] );
			}
			else
			{
				int cnt = __popc( mask );
				if ( sp + cnt > FIND_STACK )
				{
					if ( lane == 0 )
						atomicOr( &w.sc->error, ERR_TREE );
					break;
				}
				if ( ov )
					stk[sp + __popc( mask & below )] = ( ( level - 1 ) << 26 ) | child;
				sp += cnt;
			}
			__syncwarp();
		}
		__syncwarp();
	}
}

__global__ void k_clamp_pairs( DWorld w )
{
	if ( w.sc->newPairCount > w.pairCap )
		w.sc->newPairCount = w.pairCap;
}

// ---------------------------------------------------------------------------
// contact creation (contact.c:186-330) in the reference's order: row r of the
// sorted keys, decoded into (creating proxy's shape, other shape)
// ---------------------------------------------------------------------------
__device__ __forceinline__ int plan_lookup( const DWorld& w, unsigned long long key )
{
	int lo = 0, hi = w.sc->planCount - 1;
	while ( lo <= hi )
	{
		int mid = ( lo + hi ) >> 1;
		unsigned long long k = w.planKeys[mid];
		if ( k == key )
			return w.planIds[mid];
		if ( k < key )
			lo = mid + 1;
		else
			hi = mid - 1;
	}
	return -1;
}

__global__ void k_create_contacts( DWorld w, int planMode )
{
	int n = w.sc->newPairCount;
	int F = w.sc->contactFreeCount;
	int base = w.sc->contactIdCount;
	for ( int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x )
	{
		int s1 = w.pairValAlt[r], s2 = w.pairVal[r];
		unsigned long long key = pair_key( s1, s2 );
		// A is the shape with the smaller proxy key (broad_phase.c:258-267)
		int a = s1, b = s2;
		if ( w.proxyKey[s2] < w.proxyKey[s1] )
		{
			a = s2;
			b = s1;
		}
		int ta = shape_type( w.sflags[a] ), tb = shape_type( w.sflags[b] );
		bool primary;
		int id;
		if ( planMode )
		{
			// parity mode: the plan names each pair's contact id
			id = plan_lookup( w, key );
			w.newPairId[r] = id;
			if ( id < 0 )
			{
				atomicOr( &w.sc->error, ERR_PLAN_MISMATCH );
				continue;
			}
		}
		else
			id = r < F ? w.contactFree[F - 1 - r] : base + ( r - F );
		if ( id >= w.contactCap )
		{
			atomicOr( &w.sc->error, ERR_CONTACT_CAPACITY );
			continue;
		}
		if ( !registered( ta, tb, &primary ) )
			continue; // no manifold function (e.g. segment-segment): no contact
		if ( !primary )
		{
			int t = a;
			a = b;
			b = t;
		}
		int fa = w.sflags[a], fb = w.sflags[b];
		w.cshape[id] = make_int2( a, b );
		w.cbody[id] = make_int2( w.shapeBody[a], w.shapeBody[b] );
		int flags = CF_USED;
		if ( ( fa | fb ) & SF_CONTACT_EVENTS )
			flags |= CF_EVENTS;
		if ( ( fa | fb ) & SF_PRESOLVE )
			flags |= CF_PRESOLVE;
		w.cflags[id] = flags;
		w.ccolor[id] = F2D_NULL;
		w.coverflowIndex[id] = F2D_NULL;
		w.cstamp[id] = w.sc->stampBase + (unsigned long long)r;
		float4 ma = w.mat[a], mb = w.mat[b];
		// world.c:88-98 default mixing
		w.cmat[id] = make_float4( sqrtf( ma.x * mb.x ), ma.y > mb.y ? ma.y : mb.y, 0.0f, 0.0f );
		w.cmass[id] = make_float4( 0.0f, 0.0f, 0.0f, 0.0f );
		w.mnorm[id] = make_float4( 0.0f, 0.0f, 0.0f, __int_as_float( 0 ) );
		w.csimplex[id] = make_int2( 0, 0 );
		for ( int k = 0; k < 2; ++k )
		{
			w.mpA[2 * id + k] = make_float4( 0.0f, 0.0f, 0.0f, 0.0f );
			w.mpB[2 * id + k] = make_float4( 0.0f, 0.0f, 0.0f, __int_as_float( 0 ) );
			w.mpI[2 * id + k] = make_float4( 0.0f, 0.0f, 0.0f, 0.0f );
		}
	}
}

// advance the id pool after creation and clear the move flags
__global__ void k_after_create( DWorld w, int planMode )
{
	if ( blockIdx.x == 0 && threadIdx.x == 0 )
	{
		int n = w.sc->newPairCount;
		if ( planMode )
		{
			// plan ids are explicit; raise the high-water mark and drop used
			// ids from the free stack (order of the remaining ids is kept)
			int hi = w.sc->contactIdCount;
			for ( int r = 0; r < n && r < w.pairCap; ++r )
				hi = max( hi, w.newPairId[r] + 1 );
			int F = w.sc->contactFreeCount;
			int keep = 0;
			for ( int k = 0; k < F; ++k )
			{
				int id = w.contactFree[k];
				bool used = ( w.cflags[id] & CF_USED ) != 0;
				if ( !used )
					w.contactFree[keep++] = id;
			}
			// ids skipped between the old and the new high-water mark are free
			for ( int id = w.sc->contactIdCount; id < hi; ++id )
				if ( ( w.cflags[id] & CF_USED ) == 0 && keep < w.contactCap )
					w.contactFree[keep++] = id;
			w.sc->contactFreeCount = keep;
			w.sc->contactIdCount = min( hi, w.contactCap );
		}
		else
		{
			int F = w.sc->contactFreeCount;
			if ( n <= F )
				w.sc->contactFreeCount = F - n;
			else
			{
				w.sc->contactFreeCount = 0;
				w.sc->contactIdCount = min( w.sc->contactIdCount + ( n - F ), w.contactCap );
			}
		}
		w.sc->stampBase += (unsigned long long)n;
		w.sc->newPairCount = 0;
		w.sc->planCount = 0;
		w.sc->moveArrayCount = 0; // broad_phase.c:456-458: the move buffer is reset
	}
	for ( int s = blockIdx.x * blockDim.x + threadIdx.x; s < w.shapeCount; s += gridDim.x * blockDim.x )
		w.sflags[s] &= ~SF_MOVED;
}

// ---------------------------------------------------------------------------
// host driver
// ---------------------------------------------------------------------------
void launch_broadphase( DWorld& w, StepScratch& s, cudaStream_t st, int planMode, HostHook pairHook,
						void* hookContext )
{
	int gridS = grid_for( w.shapeCount );
	launch_pt_host_moves( w, s, st );
	// the pair hash of the live contacts is built beside the leaf ordering,
	// which does not touch it; both meet before the refit
	cudaStream_t hs = s.side[0] ? s.side[0] : st;
	if ( hs != st )
	{
		cudaEventRecord( s.sideFork, st );
		cudaStreamWaitEvent( hs, s.sideFork, 0 );
	}
	k_hash_clear<<<grid_for( w.hashCap ), BP_THREADS, 0, hs>>>( w );
	k_hash_insert<<<grid_for( w.contactCap ), BP_THREADS, 0, hs>>>( w );
	if ( hs != st )
		cudaEventRecord( s.sideJoin[0], hs );
	k_leaf_flags<<<gridS, BP_THREADS, 0, st>>>( w, s.tmpA );
	scan_lookback( s.tmpA, s.tmpB, nullptr, w.shapeCount, w.shapeCap, &w.sc->treeLeafCount, s.scanState, &w.sc->error,
				   st, &w.sc->rebuildOrder );
	k_leaf_compact<<<gridS, BP_THREADS, 0, st>>>( w, s.tmpA, s.tmpB );
	k_bounds_partial<<<s.boundsBlocks, BP_THREADS, 0, st>>>( w, s.bounds );
	k_bounds_final<<<1, BP_THREADS, 0, st>>>( &w.sc->rebuildOrder, s.bounds, s.boundsBlocks );
	k_morton<<<gridS, BP_THREADS, 0, st>>>( w, s.bounds );
	sort_coop<unsigned>( w.mortonKeys, w.leafShape, w.mortonKeysAlt, w.leafShapeAlt, &w.sc->treeLeafCount, 30,
						 w.sortHist, &w.sc->barrierCount, &w.sc->error, s.sortBlocks32, st, &w.sc->rebuildOrder );
	if ( hs != st )
		cudaStreamWaitEvent( st, s.sideJoin[0], 0 );
	k_wide_refit<<<( ( w.shapeCap + WIDE - 1 ) / WIDE + 7 ) / 8, BP_THREADS, 0, st>>>( w );
	k_find_pairs<<<( w.shapeCap + FIND_WARPS - 1 ) / FIND_WARPS, BP_THREADS, 0, st>>>( w );
	k_clamp_pairs<<<1, 1, 0, st>>>( w );
	// keys are unique (one per pair), so the key order alone fixes the result
	int bits = 2 * w.pairKeyBits + 2;
	sort_coop<unsigned long long>( w.pairKeys, w.pairVal, w.pairKeysAlt, w.pairValAlt, &w.sc->newPairCount, bits,
								   w.sortHist, &w.sc->barrierCount, &w.sc->error, s.sortBlocks64, st );
	launch_pt_decode( w, st );
	// world.c:488-502: the dynamic and kinematic trees are rebuilt over
	// their enlarged nodes every step, once the new pairs have their tree
	// ranks, beside the rest of the collide phase (as the reference's rebuild
	// task runs beside its collide tasks); nothing until the solver reads or
	// writes them, and the world joins the rebuild's stream before its
	// persistent cooperative solver, which needs the whole GPU
	if ( s.rebuild )
	{
		cudaEventRecord( s.rebuildFork, st );
		cudaStreamWaitEvent( s.rebuild, s.rebuildFork, 0 );
		if ( s.rebuildT0 )
			cudaEventRecord( s.rebuildT0, s.rebuild );
		launch_pt_rebuild( w, s, s.rebuild );
		if ( s.rebuildT1 )
			cudaEventRecord( s.rebuildT1, s.rebuild );
		cudaEventRecord( s.rebuildJoin, s.rebuild );
	}
	else
		launch_pt_rebuild( w, s, st );
	// broad_phase.c:267-278: the custom filter sees the new pairs last
	if ( pairHook )
		pairHook( hookContext );
	k_create_contacts<<<grid_for( w.pairCap ), BP_THREADS, 0, st>>>( w, planMode );
	if ( w.isl )
		launch_isl_new_contacts( w, s, st, planMode );
	k_after_create<<<gridS, BP_THREADS, 0, st>>>( w, planMode );
}
