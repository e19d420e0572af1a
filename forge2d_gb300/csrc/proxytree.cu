// The reference's broadphase trees on the device, and the move array.
//
// Box2D v3.1.1 creates a step's new contacts proxy by proxy in move-array
// order, each proxy's pairs by tree (dynamic, static, kinematic) and within
// a tree left to right (broad_phase.c:311-474: each query visits leaves
// depth first, child2's subtree first, and prepends every pair to the
// proxy's list). That order fixes contact ids, colours and the Gauss-Seidel
// order, so this file keeps the reference's own trees (dynamic_tree.c) node
// for node and turns their topology into a sort key:
//
//   * move array (solver.c:1842-1905): the proxies enlarged by the finalize
//     pass, awake bodies in awake-set order and each body's shapes in list
//     order, then the proxies the host buffered between steps (creation,
//     transforms) in call order, each proxy once;
//   * enlarge (dynamic_tree.c:827-866): one thread per enlarged proxy grows
//     its ancestors' boxes with compare-and-swap, stopping at an ancestor
//     that already held the box and was already marked, which yields the
//     reference's boxes (old box union every new leaf box below) and marks;
//   * partial rebuild (dynamic_tree.c:1872-1989, b2PartitionMid :1426):
//     every enlarged internal node is freed in pre-order and the nodes below
//     them (leaves and intact subtrees) are gathered left to right; the
//     median-split build over them runs level by level. The reference's
//     Hoare partition has a closed form: with L centres below the pivot, the
//     k-th centre of [0, L) that is not below swaps with the k-th centre of
//     [L, n) that is, counted from the end. Large segments are partitioned
//     by the whole grid (one cooperative launch, chunk counts and offsets
//     between grid barriers), segments of at most PT_SMALL nodes by one
//     block in shared memory, a warp per sub-segment. The build allocates
//     its nodes in pre-order from the LIFO free list, so the node of a
//     segment [s, e) reached through c child1 edges is freed[F - 1 - s - c]
//     (F internal nodes; s + c is its pre-order index);
//   * ranks: a leaf's left-to-right position is the sum of the child1 leaf
//     counts along its path (found per new pair in broadphase.cu); a new
//     pair's key is (move index of the proxy whose query creates it, tree,
//     rank of the other proxy). Every leaf's rank is kept only for the
//     static tree (continuous collision visits static shapes in its order),
//     recomputed when the host uploads a tree.
#include "dscan.cuh"
#include "dsort.cuh"
#include "dsync.cuh"
#include "dworld.cuh"
#include "kernels.cuh"

#include <climits>

#define PT_THREADS 256
#define PT_SMALL 1024
#define PT_CHUNK 1024
#define PT_ITEMS ( PT_CHUNK / PT_THREADS )
#define PT_WARPS ( PT_THREADS / 32 )
#define PT_GUARD ( 1 << 16 )

__device__ __forceinline__ int pt_atom_add( int* p, int v )
{
	int old;
	asm volatile( "atom.acq_rel.gpu.global.add.s32 %0, [%1], %2;" : "=r"( old ) : "l"( p ), "r"( v ) : "memory" );
	return old;
}

// float -> int with the same order (exact min / max through integer atomics)
__device__ __forceinline__ int f2o( float f )
{
	int i = __float_as_int( f );
	return i >= 0 ? i : i ^ 0x7fffffff;
}

__device__ __forceinline__ float o2f( int i )
{
	return __int_as_float( i >= 0 ? i : i ^ 0x7fffffff );
}

// b2AABB_Union with the reference's tie rule (the second operand wins ties)
__device__ __forceinline__ float4 pt_union( float4 a, float4 b )
{
	return make_float4( a.x < b.x ? a.x : b.x, a.y < b.y ? a.y : b.y, a.z > b.z ? a.z : b.z, a.w > b.w ? a.w : b.w );
}

__device__ __forceinline__ bool cas_lower( float* addr, float v )
{
	int* ia = (int*)addr;
	int old = *(volatile int*)ia;
	while ( v < __int_as_float( old ) )
	{
		int prev = atomicCAS( ia, old, __float_as_int( v ) );
		if ( prev == old )
			return true;
		old = prev;
	}
	return false;
}

__device__ __forceinline__ bool cas_upper( float* addr, float v )
{
	int* ia = (int*)addr;
	int old = *(volatile int*)ia;
	while ( __int_as_float( old ) < v )
	{
		int prev = atomicCAS( ia, old, __float_as_int( v ) );
		if ( prev == old )
			return true;
		old = prev;
	}
	return false;
}

// dynamic_tree.c:827-866 b2DynamicTree_EnlargeProxy, one proxy of many at
// once (see the file comment)
__device__ void pt_enlarge( const DProxyTree& T, int leaf, float4 b, int* err )
{
	T.box[leaf] = b;
	int p = T.parent[leaf];
	for ( int guard = 0; p >= 0; ++guard )
	{
		if ( guard > PT_GUARD )
		{
			atomicOr( err, ERR_TREE );
			return;
		}
		float* f = (float*)( T.box + p );
		bool changed = cas_lower( f + 0, b.x );
		changed |= cas_lower( f + 1, b.y );
		changed |= cas_upper( f + 2, b.z );
		changed |= cas_upper( f + 3, b.w );
		int old = atomicOr( T.flags + p, PT_ENLARGED );
		if ( !changed && ( old & PT_ENLARGED ) )
			return;
		p = *(volatile int*)( T.parent + p );
	}
}

// ---------------------------------------------------------------------------
// move array
// ---------------------------------------------------------------------------
__device__ __forceinline__ bool body_awake_plain( int f )
{
	return ( f & ( BF_USED | BF_ENABLED ) ) == ( BF_USED | BF_ENABLED ) && body_type( f ) != 0 && ( f & BF_ASLEEP ) == 0;
}

// per awake-set position: the body's enlarged shapes
__global__ void k_pt_move_count( DWorld w, int* cnt )
{
	int n = w.isl ? w.isl->awakeBodyCount : w.sc->awakeOrderCount;
	if ( blockIdx.x == 0 && threadIdx.x == 0 )
		w.sc->fastCount = 0;
	for ( int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x )
	{
		int b = w.isl ? w.isl->awakeBodies[k] : w.awakeOrder[k];
		int c = 0;
		if ( w.isl || body_awake_plain( w.bflags[b] ) )
			for ( int s = w.headShape[b], guard = 0; s != F2D_NULL && guard < ( 1 << 20 ); s = w.nextShape[s], ++guard )
				c += ( w.sflags[s] & SF_ENLARGED ) ? 1 : 0;
		cnt[k] = c;
	}
}

// move-array slots in awake order; the proxies' tree leaves are enlarged
__global__ void k_pt_move_assign( DWorld w, const int* pos )
{
	int n = w.isl ? w.isl->awakeBodyCount : w.sc->awakeOrderCount;
	for ( int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x )
	{
		int b = w.isl ? w.isl->awakeBodies[k] : w.awakeOrder[k];
		if ( !w.isl && !body_awake_plain( w.bflags[b] ) )
			continue;
		int slot = pos[k];
		for ( int s = w.headShape[b], guard = 0; s != F2D_NULL && guard < ( 1 << 20 ); s = w.nextShape[s], ++guard )
		{
			int f = w.sflags[s];
			if ( ( f & SF_ENLARGED ) == 0 )
				continue;
			w.moveShape[slot] = s;
			w.shapeMove[s] = slot;
			slot += 1;
			w.sflags[s] = ( f & ~SF_ENLARGED ) | SF_MOVED;
			int pk = w.proxyKey[s];
			pt_enlarge( w.pt[pk & 3], pk >> 2, w.fat[s], &w.sc->error );
		}
	}
}

// the host's buffered proxies follow, skipping those already in the array
__global__ void k_pt_host_flags( DWorld w, int* flag )
{
	int n = w.sc->hostMoveCount;
	for ( int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x )
	{
		int s = w.hostMoves[i];
		int f = w.sflags[s];
		flag[i] = ( f & ( SF_USED | SF_PROXY | SF_MOVED ) ) == ( SF_USED | SF_PROXY ) ? 1 : 0;
	}
}

__global__ void k_pt_host_write( DWorld w, const int* flag, const int* pos )
{
	int n = w.sc->hostMoveCount;
	int base = w.sc->moveArrayCount;
	for ( int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x )
	{
		if ( flag[i] == 0 )
			continue;
		int s = w.hostMoves[i];
		int slot = base + pos[i];
		w.moveShape[slot] = s;
		w.shapeMove[s] = slot;
		w.sflags[s] |= SF_MOVED;
	}
}

__global__ void k_pt_host_done( DWorld w, const int* flag, const int* pos )
{
	int n = w.sc->hostMoveCount;
	if ( n > 0 )
		w.sc->moveArrayCount += pos[n - 1] + flag[n - 1];
	w.sc->hostMoveCount = 0;
}

// ---------------------------------------------------------------------------
// new-pair keys -> the creating proxy's shape (the other shape is the
// sorted value)
// ---------------------------------------------------------------------------
__global__ void k_pt_decode( DWorld w )
{
	int n = min( w.sc->newPairCount, w.pairCap );
	int rb = w.pairKeyBits;
	for ( int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x )
		w.pairValAlt[r] = w.moveShape[(int)( w.pairKeys[r] >> ( rb + 2 ) )];
}

// ---------------------------------------------------------------------------
// partial rebuild
// ---------------------------------------------------------------------------
__global__ void k_pt_mark( DWorld w, int t )
{
	const DProxyTree T = w.pt[t];
	const DRebuild R = w.rb;
	for ( int i = blockIdx.x * blockDim.x + threadIdx.x; i < T.cap; i += gridDim.x * blockDim.x )
	{
		int f = T.flags[i];
		R.doomed[i] = ( f & ( PT_ALLOCATED | PT_LEAF | PT_ENLARGED ) ) == ( PT_ALLOCATED | PT_ENLARGED ) ? 1 : 0;
		R.cnt[i] = 0;
	}
	if ( blockIdx.x == 0 && threadIdx.x == 0 )
	{
		int root = w.sc->treeRoot[t];
		int active = 0;
		if ( root >= 0 )
			active = ( T.flags[root] & ( PT_ALLOCATED | PT_LEAF | PT_ENLARGED ) ) == ( PT_ALLOCATED | PT_ENLARGED );
		w.sc->rbActive = active;
		w.sc->rbCount = 0;
		w.sc->rbLarge[0] = 0;
		w.sc->rbLarge[1] = 0;
		w.sc->rbSmall = 0;
		w.sc->rbRefresh = 0;
	}
}

// gathered nodes below each doomed node: the second child to arrive sums
__global__ void k_pt_count( DWorld w, int t )
{
	if ( w.sc->rbActive == 0 )
		return;
	const DProxyTree T = w.pt[t];
	const DRebuild R = w.rb;
	int root = w.sc->treeRoot[t];
	for ( int i = blockIdx.x * blockDim.x + threadIdx.x; i < T.cap; i += gridDim.x * blockDim.x )
	{
		if ( ( T.flags[i] & PT_ALLOCATED ) == 0 || R.doomed[i] )
			continue;
		int p = T.parent[i];
		if ( p < 0 || R.doomed[p] == 0 )
			continue;
		int c = i;
		for ( int guard = 0;; ++guard )
		{
			if ( guard > PT_GUARD )
			{
				atomicOr( &w.sc->error, ERR_TREE );
				break;
			}
			p = T.parent[c];
			if ( p < 0 || p >= T.cap )
			{
				atomicOr( &w.sc->error, ERR_TREE );
				break;
			}
			if ( pt_atom_add( R.cnt + p, 1 ) == 0 )
				break;
			int a = T.child1[p], b = T.child2[p];
			int va = R.doomed[a] ? __ldcg( R.rlc + a ) : 1;
			int vb = R.doomed[b] ? __ldcg( R.rlc + b ) : 1;
			__stcg( R.rlc + p, va + vb );
			__threadfence();
			if ( p == root )
				break;
			c = p;
		}
	}
}

// left-to-right position of each gathered node, pre-order position of each
// doomed node (the free order)
__global__ void k_pt_gather( DWorld w, int t )
{
	if ( w.sc->rbActive == 0 )
		return;
	const DProxyTree T = w.pt[t];
	const DRebuild R = w.rb;
	int root = w.sc->treeRoot[t];
	for ( int i = blockIdx.x * blockDim.x + threadIdx.x; i < T.cap; i += gridDim.x * blockDim.x )
	{
		if ( ( T.flags[i] & PT_ALLOCATED ) == 0 )
			continue;
		bool dm = R.doomed[i] != 0;
		int pi = T.parent[i];
		bool gathered = !dm && pi >= 0 && R.doomed[pi] != 0;
		if ( !dm && !gathered )
			continue;
		int acc = 0, c1 = 0, c = i;
		bool ok = true;
		for ( int guard = 0; c != root; ++guard )
		{
			int p = T.parent[c];
			if ( guard > PT_GUARD || p < 0 || p >= T.cap )
			{
				atomicOr( &w.sc->error, ERR_TREE );
				ok = false;
				break;
			}
			if ( T.child2[p] == c )
			{
				int a = T.child1[p];
				acc += R.doomed[a] ? R.rlc[a] : 1;
			}
			else
				c1 += 1;
			c = p;
		}
		int total = R.rlc[root];
		if ( !ok || ( dm ? acc + c1 >= total - 1 : acc >= total ) )
		{
			atomicOr( &w.sc->error, ERR_TREE );
			continue;
		}
		if ( dm )
		{
			R.freed[acc + c1] = i;
			R.cnt[i] = 0;
		}
		else
		{
			float4 b = T.box[i];
			R.gIdx[acc] = i;
			R.gCen[acc] = make_float2( 0.5f * ( b.x + b.z ), 0.5f * ( b.y + b.w ) );
		}
	}
	if ( blockIdx.x == 0 && threadIdx.x == 0 )
	{
		int n = R.rlc[root];
		if ( n < 2 || n > T.cap )
		{
			atomicOr( &w.sc->error, ERR_TREE );
			w.sc->rbActive = 0;
			return;
		}
		w.sc->rbCount = n;
		if ( n <= PT_SMALL )
		{
			R.segSmall[0] = make_int4( 0, n, 0, 0 );
			w.sc->rbSmall = 1;
		}
		else
		{
			R.segA[0] = make_int4( 0, n, 0, 0 );
			R.segBounds[0] = R.segBounds[1] = INT_MAX;
			R.segBounds[2] = R.segBounds[3] = INT_MIN;
			R.segBelow[0] = 0;
			w.sc->rbLarge[0] = 1;
		}
	}
}

__device__ __forceinline__ int pt_find( const int* base, int count, int x )
{
	int lo = 0, hi = count - 1;
	while ( lo < hi )
	{
		int mid = ( lo + hi + 1 ) >> 1;
		if ( __ldcg( base + mid ) <= x )
			lo = mid;
		else
			hi = mid - 1;
	}
	return lo;
}

// the same search over a shared-memory array
__device__ __forceinline__ int pt_find_s( const int* base, int count, int x )
{
	int lo = 0, hi = count - 1;
	while ( lo < hi )
	{
		int mid = ( lo + hi + 1 ) >> 1;
		if ( base[mid] <= x )
			lo = mid;
		else
			hi = mid - 1;
	}
	return lo;
}

__device__ __forceinline__ float pt_axis( float2 c, bool axisY )
{
	return axisY ? c.y : c.x;
}

// pivot of b2PartitionMid from the segment's centre bounds
__device__ __forceinline__ float pt_pivot( const int* bounds, bool* axisY )
{
	float lx = o2f( __ldcg( bounds + 0 ) ), ly = o2f( __ldcg( bounds + 1 ) );
	float hx = o2f( __ldcg( bounds + 2 ) ), hy = o2f( __ldcg( bounds + 3 ) );
	float dx = hx - lx, dy = hy - ly;
	*axisY = !( dx > dy );
	return *axisY ? 0.5f * ( ly + hy ) : 0.5f * ( lx + hx );
}

__device__ __forceinline__ int block_sum( int v, int* red )
{
	int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
	for ( int o = 16; o > 0; o >>= 1 )
		v += __shfl_xor_sync( 0xffffffffu, v, o );
	__syncthreads();
	if ( lane == 0 )
		red[wid] = v;
	__syncthreads();
	int s = 0;
	for ( int k = 0; k < PT_WARPS; ++k )
		s += red[k];
	return s;
}

__device__ __forceinline__ int block_excl( int v, int* red, int* total )
{
	int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
	int x = v;
#pragma unroll
	for ( int o = 1; o < 32; o <<= 1 )
	{
		int y = __shfl_up_sync( 0xffffffffu, x, o );
		if ( lane >= o )
			x += y;
	}
	__syncthreads();
	if ( lane == 31 )
		red[wid] = x;
	__syncthreads();
	int before = 0, all = 0;
	for ( int k = 0; k < PT_WARPS; ++k )
	{
		if ( k < wid )
			before += red[k];
		all += red[k];
	}
	*total = all;
	return before + x - v;
}

// Median-split levels of the segments larger than PT_SMALL: one cooperative
// launch, the whole grid on each level, four grid barriers a level:
//   A  every block derives the level's segments from the last level's
//      splits (deterministic, in shared memory), links the last level's
//      nodes (its share of them), and accumulates the centre bounds;
//   B  centres below each pivot, per chunk;
//   C  each misplaced centre's rank: left of the split and not below from
//      the left, right of it and below from the right (chunk offsets follow
//      from the per-chunk counts, as only the chunk holding the split mixes
//      both sides);
//   D  the k-th misplaced left centre swaps with the k-th misplaced right one
//      (b2PartitionMid's swaps in closed form).
// Accumulators are double-buffered by level parity; a level resets the next
// level's after its last reader has passed a barrier.
#define PT_LMAX 2048
struct PtLarge
{
	int4 seg[2][PT_LMAX];
	int chunkBase[PT_LMAX + 1];
	int pairBase[PT_LMAX + 1];
	int red[4 * PT_WARPS];
	int count[2];
};

// exclusive prefix of vals[0..L) into out[0..L] (out[L] = total), whole block
template <typename F>
__device__ __forceinline__ void pt_block_prefix( int L, F value, int* out, int* red )
{
	int carry = 0;
	for ( int base = 0; base < L; base += PT_THREADS )
	{
		int j = base + threadIdx.x;
		int v = j < L ? value( j ) : 0;
		int total;
		int ex = block_excl( v, red, &total );
		if ( j < L )
			out[j] = carry + ex;
		carry += total;
		__syncthreads();
	}
	if ( threadIdx.x == 0 )
		out[L] = carry;
	__syncthreads();
}

__device__ __forceinline__ int pt_split( int n, int below )
{
	return ( below == 0 || below == n ) ? n / 2 : below;
}

__global__ void __launch_bounds__( PT_THREADS ) k_pt_large( DWorld w, int t, unsigned* counter )
{
	extern __shared__ __align__( 16 ) unsigned char ptSmemL[];
	PtLarge& sm = *reinterpret_cast<PtLarge*>( ptSmemL );
	DScalars* sc = w.sc;
	if ( __ldcg( &sc->rbActive ) == 0 || __ldcg( &sc->rbLarge[0] ) == 0 )
		return;
	const DProxyTree T = w.pt[t];
	const DRebuild R = w.rb;
	const int tid = threadIdx.x;
	const int F = __ldcg( &sc->rbCount ) - 1;
	const int SC = R.segCap;
	unsigned epoch = 0;
	if ( tid == 0 )
	{
		sm.seg[0][0] = __ldcg( R.segA );
		sm.count[0] = 1;
	}
	__syncthreads();
	for ( int level = 0; level < 64; ++level )
	{
		const int cur = level & 1, prv = cur ^ 1;
		int* bounds = R.segBounds + 4 * SC * cur;
		int* belowAcc = R.segBelow + SC * cur;
		// ---- A: this level's segments, the last level's links, bounds ----
		if ( level > 0 )
		{
			const int Lp = sm.count[prv];
			const int* belowPrev = R.segBelow + SC * prv;
			pt_block_prefix(
				Lp,
				[&]( int j ) {
					int4 sg = sm.seg[prv][j];
					int n = sg.y - sg.x, split = pt_split( n, __ldcg( belowPrev + j ) );
					return ( split > PT_SMALL ? 1 : 0 ) + ( n - split > PT_SMALL ? 1 : 0 );
				},
				sm.pairBase, sm.red );
			for ( int j = tid; j < Lp; j += PT_THREADS )
			{
				int4 sg = sm.seg[prv][j];
				int n = sg.y - sg.x, split = pt_split( n, __ldcg( belowPrev + j ) );
				int o = sm.pairBase[j];
				if ( o + 2 > PT_LMAX )
					continue;
				if ( split > PT_SMALL )
					sm.seg[cur][o++] = make_int4( sg.x, sg.x + split, sg.z + 1, 0 );
				if ( n - split > PT_SMALL )
					sm.seg[cur][o] = make_int4( sg.x + split, sg.y, sg.z, 0 );
			}
			if ( tid == 0 )
				sm.count[cur] = sm.pairBase[Lp];
			// link the last level's nodes (this block's share)
			for ( int j = blockIdx.x * PT_THREADS + tid; j < Lp; j += gridDim.x * PT_THREADS )
			{
				int4 sg = sm.seg[prv][j];
				int n = sg.y - sg.x, split = pt_split( n, __ldcg( belowPrev + j ) );
				int c1 = sg.z;
				int node = R.freed[F - 1 - ( sg.x + c1 )];
				int ls = sg.x, le = sg.x + split, re = sg.y;
				int left = le - ls == 1 ? __ldcg( R.gIdx + ls ) : R.freed[F - 1 - ( ls + c1 + 1 )];
				int right = re - le == 1 ? __ldcg( R.gIdx + le ) : R.freed[F - 1 - ( le + c1 )];
				T.child1[node] = left;
				T.child2[node] = right;
				T.parent[left] = node;
				T.parent[right] = node;
				// children the bottom-up pass starts from: single gathered nodes
				// and the roots of small segments (k_pt_small does their inside)
				if ( le - ls <= PT_SMALL )
					__stcg( R.rfStart + atomicAdd( &sc->rbRefresh, 1 ), left );
				if ( re - le <= PT_SMALL )
					__stcg( R.rfStart + atomicAdd( &sc->rbRefresh, 1 ), right );
				if ( le - ls >= 2 && le - ls <= PT_SMALL )
					__stcg( R.segSmall + atomicAdd( &sc->rbSmall, 1 ), make_int4( ls, le, c1 + 1, 0 ) );
				if ( re - le >= 2 && re - le <= PT_SMALL )
					__stcg( R.segSmall + atomicAdd( &sc->rbSmall, 1 ), make_int4( le, re, c1, 0 ) );
			}
			__syncthreads();
			if ( sm.pairBase[Lp] > PT_LMAX )
			{
				if ( blockIdx.x == 0 && tid == 0 )
					atomicOr( &sc->error, ERR_TREE );
				return;
			}
		}
		const int L = sm.count[cur];
		if ( L == 0 )
			return; // all blocks see the same count
		pt_block_prefix(
			L, [&]( int j ) { return ( sm.seg[cur][j].y - sm.seg[cur][j].x + PT_CHUNK - 1 ) / PT_CHUNK; },
			sm.chunkBase, sm.red );
		const int C = sm.chunkBase[L];
		for ( int c = blockIdx.x; c < C; c += gridDim.x )
		{
			int j = pt_find_s( sm.chunkBase, L, c );
			int4 sg = sm.seg[cur][j];
			int lo = sg.x + ( c - sm.chunkBase[j] ) * PT_CHUNK, hi = min( sg.y, lo + PT_CHUNK );
			int mnx = INT_MAX, mny = INT_MAX, mxx = INT_MIN, mxy = INT_MIN;
			for ( int i = lo + tid; i < hi; i += PT_THREADS )
			{
				float2 cc = __ldcg( R.gCen + i );
				mnx = min( mnx, f2o( cc.x ) );
				mny = min( mny, f2o( cc.y ) );
				mxx = max( mxx, f2o( cc.x ) );
				mxy = max( mxy, f2o( cc.y ) );
			}
#pragma unroll
			for ( int o = 16; o > 0; o >>= 1 )
			{
				mnx = min( mnx, __shfl_xor_sync( 0xffffffffu, mnx, o ) );
				mny = min( mny, __shfl_xor_sync( 0xffffffffu, mny, o ) );
				mxx = max( mxx, __shfl_xor_sync( 0xffffffffu, mxx, o ) );
				mxy = max( mxy, __shfl_xor_sync( 0xffffffffu, mxy, o ) );
			}
			if ( ( tid & 31 ) == 0 )
			{
				atomicMin( bounds + 4 * j + 0, mnx );
				atomicMin( bounds + 4 * j + 1, mny );
				atomicMax( bounds + 4 * j + 2, mxx );
				atomicMax( bounds + 4 * j + 3, mxy );
			}
		}
		if ( !grid_barrier( counter, &sc->error, epoch ) )
			return;
		// ---- B: centres below the pivot per chunk; next level's accumulators ----
		if ( blockIdx.x == 0 )
		{
			int* nb = R.segBounds + 4 * SC * prv;
			int* nbl = R.segBelow + SC * prv;
			int lim = min( 2 * L, SC );
			for ( int j = tid; j < lim; j += PT_THREADS )
			{
				__stcg( nb + 4 * j + 0, INT_MAX );
				__stcg( nb + 4 * j + 1, INT_MAX );
				__stcg( nb + 4 * j + 2, INT_MIN );
				__stcg( nb + 4 * j + 3, INT_MIN );
				__stcg( nbl + j, 0 );
			}
		}
		for ( int c = blockIdx.x; c < C; c += gridDim.x )
		{
			int j = pt_find_s( sm.chunkBase, L, c );
			int4 sg = sm.seg[cur][j];
			int lo = sg.x + ( c - sm.chunkBase[j] ) * PT_CHUNK, hi = min( sg.y, lo + PT_CHUNK );
			bool axisY;
			float pivot = pt_pivot( bounds + 4 * j, &axisY );
			int below = 0;
			for ( int i = lo + tid; i < hi; i += PT_THREADS )
				below += pt_axis( __ldcg( R.gCen + i ), axisY ) < pivot ? 1 : 0;
			below = block_sum( below, sm.red );
			if ( tid == 0 )
			{
				__stcg( R.chunkStat + c, below );
				atomicAdd( belowAcc + j, below );
			}
		}
		if ( !grid_barrier( counter, &sc->error, epoch ) )
			return;
		// ---- C: ranks of the misplaced centres ----
		for ( int c = blockIdx.x; c < C; c += gridDim.x )
		{
			int j = pt_find_s( sm.chunkBase, L, c );
			int4 sg = sm.seg[cur][j];
			int c0 = sm.chunkBase[j], cEnd = sm.chunkBase[j + 1];
			int lo = sg.x + ( c - c0 ) * PT_CHUNK, hi = min( sg.y, lo + PT_CHUNK );
			bool axisY;
			float pivot = pt_pivot( bounds + 4 * j, &axisY );
			int m = sg.x + __ldcg( belowAcc + j );
			// every chunk before this one lies left of the split when this one
			// holds misplaced left centres; every later one right of it when
			// this one holds misplaced right centres
			int offL = 0, offR = 0;
			if ( lo < m )
				for ( int k = c0 + tid; k < c; k += PT_THREADS )
				{
					int klo = sg.x + ( k - c0 ) * PT_CHUNK, khi = min( sg.y, klo + PT_CHUNK );
					offL += ( khi - klo ) - __ldcg( R.chunkStat + k );
				}
			if ( hi > m )
				for ( int k = c + 1 + tid; k < cEnd; k += PT_THREADS )
					offR += __ldcg( R.chunkStat + k );
			offL = block_sum( offL, sm.red );
			offR = block_sum( offR, sm.red + PT_WARPS );
			int first = lo + tid * PT_ITEMS;
			int fl = 0, fr = 0;
			int kind[PT_ITEMS];
#pragma unroll
			for ( int k = 0; k < PT_ITEMS; ++k )
			{
				int i = first + k;
				kind[k] = 0;
				if ( i < hi )
				{
					bool below = pt_axis( __ldcg( R.gCen + i ), axisY ) < pivot;
					if ( i < m && !below )
						kind[k] = 1;
					else if ( i >= m && below )
						kind[k] = 2;
				}
				fl += kind[k] == 1;
				fr += kind[k] == 2;
			}
			int totL, totR;
			int exL = block_excl( fl, sm.red, &totL );
			int exR = block_excl( fr, sm.red + PT_WARPS, &totR );
#pragma unroll
			for ( int k = 0; k < PT_ITEMS; ++k )
			{
				int i = first + k;
				if ( kind[k] == 1 )
				{
					__stcg( R.bl + sg.x + offL + exL, i );
					exL += 1;
				}
				else if ( kind[k] == 2 )
				{
					__stcg( R.br + sg.x + offR + ( totR - 1 - exR ), i );
					exR += 1;
				}
			}
			// the swap count: the chunk holding the split's last left centre
			// (or the first chunk when nothing is below the pivot)
			if ( tid == 0 && ( m > sg.x ? ( lo <= m - 1 && m - 1 < hi ) : c == c0 ) )
				__stcg( R.pairBase + j, m > sg.x ? offL + totL : 0 );
			__syncthreads();
		}
		if ( !grid_barrier( counter, &sc->error, epoch ) )
			return;
		// ---- D: the swaps ----
		pt_block_prefix( L, [&]( int j ) { return __ldcg( R.pairBase + j ); }, sm.pairBase, sm.red );
		{
			int P = sm.pairBase[L];
			for ( int p = blockIdx.x * PT_THREADS + tid; p < P; p += gridDim.x * PT_THREADS )
			{
				int j = pt_find_s( sm.pairBase, L, p );
				int4 sg = sm.seg[cur][j];
				int k = p - sm.pairBase[j];
				int a = __ldcg( R.bl + sg.x + k ), b = __ldcg( R.br + sg.x + k );
				int ia = __ldcg( R.gIdx + a ), ib = __ldcg( R.gIdx + b );
				float2 ca = __ldcg( R.gCen + a ), cb = __ldcg( R.gCen + b );
				__stcg( R.gIdx + a, ib );
				__stcg( R.gIdx + b, ia );
				__stcg( R.gCen + a, cb );
				__stcg( R.gCen + b, ca );
			}
		}
		if ( !grid_barrier( counter, &sc->error, epoch ) )
			return;
	}
}

// shared memory of k_pt_small (dynamic: more than the static 48 KB)
#define PT_SMALL_LEVELS 64
struct PtSmall
{
	int idx[PT_SMALL];
	int freed[PT_SMALL];
	int4 kid[PT_SMALL]; // (freed position, child1, child2, -) in creation order
	int levelStart[PT_SMALL_LEVELS + 1];
	int count[2];
	int kidCount;
	union
	{
		struct // the median-split levels
		{
			float2 cen[PT_SMALL];
			int bl[PT_SMALL];
			int br[PT_SMALL];
			int4 item[2][PT_SMALL / 2];
			int split[PT_SMALL / 2];
		} b;
		struct // the bottom-up pass: gathered nodes at their positions, then
			   // the new internal nodes at PT_SMALL + freed position
		{
			float4 box[2 * PT_SMALL];
			unsigned long long cat[2 * PT_SMALL];
			int2 hl[2 * PT_SMALL]; // height, leaves
		} r;
	} u;
};

// a new internal node from its two children (dynamic_tree.c:1990-2010)
__device__ __forceinline__ void pt_refresh_node( const DProxyTree& T, int p, int a, int b )
{
	T.box[p] = pt_union( __ldcg( T.box + a ), __ldcg( T.box + b ) );
	T.height[p] = 1 + max( __ldcg( T.height + a ), __ldcg( T.height + b ) );
	T.cat[p] = __ldcg( T.cat + a ) | __ldcg( T.cat + b );
	T.leaves[p] = __ldcg( T.leaves + a ) + __ldcg( T.leaves + b );
	T.flags[p] = PT_ALLOCATED;
}

// b2PartitionMid (dynamic_tree.c:1426) on one thread: the centre bounds,
// the pivot on the longer axis, then the Hoare partition itself (the k-th
// centre of [s, s + below) that is not below the pivot swaps with the k-th
// centre of [s + below, e) that is, counted from the end), the same pairs as
// the warp form. Returns the split (nodes on the left).
#define PT_SERIAL 32
__device__ __forceinline__ int pt_partition_serial( int* idx, float2* cen, int s, int e )
{
	int cnt = e - s;
	if ( cnt <= 2 )
		return 1;
	float lx = FLT_MAX, ly = FLT_MAX, hx = -FLT_MAX, hy = -FLT_MAX;
	for ( int i = s; i < e; ++i )
	{
		float2 c = cen[i];
		lx = c.x < lx ? c.x : lx;
		ly = c.y < ly ? c.y : ly;
		hx = c.x > hx ? c.x : hx;
		hy = c.y > hy ? c.y : hy;
	}
	float dx = hx - lx, dy = hy - ly;
	bool axisY = !( dx > dy );
	float pivot = axisY ? 0.5f * ( ly + hy ) : 0.5f * ( lx + hx );
	int below = 0;
	for ( int i = s; i < e; ++i )
		below += pt_axis( cen[i], axisY ) < pivot ? 1 : 0;
	if ( below == 0 || below == cnt )
		return cnt / 2;
	int mid = s + below, i = s, j = e - 1;
	for ( ;; )
	{
		while ( i < mid && pt_axis( cen[i], axisY ) < pivot )
			++i;
		while ( j >= mid && !( pt_axis( cen[j], axisY ) < pivot ) )
			--j;
		// as many misplaced on each side, so both run out together
		if ( i >= mid || j < mid )
			break;
		int ti = idx[i];
		idx[i] = idx[j];
		idx[j] = ti;
		float2 tc = cen[i];
		cen[i] = cen[j];
		cen[j] = tc;
		++i;
		--j;
	}
	return below;
}

__global__ void __launch_bounds__( PT_THREADS ) k_pt_small( DWorld w, int t )
{
	extern __shared__ __align__( 16 ) unsigned char ptSmem[];
	PtSmall& sm = *reinterpret_cast<PtSmall*>( ptSmem );
	int* sIdx = sm.idx;
	float2* sCen = sm.u.b.cen;
	int* sBL = sm.u.b.bl;
	int* sBR = sm.u.b.br;
	int* sFreed = sm.freed;
	int4( *sItem )[PT_SMALL / 2] = sm.u.b.item;
	int* sSplit = sm.u.b.split;
	int* sCount = sm.count;
	DScalars* sc = w.sc;
	if ( sc->rbActive == 0 )
		return;
	const DProxyTree T = w.pt[t];
	const DRebuild R = w.rb;
	const int S = sc->rbSmall;
	const int F = sc->rbCount - 1;
	const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
	const unsigned lt = ( 1u << lane ) - 1u;
	for ( int q = blockIdx.x; q < S; q += gridDim.x )
	{
		int4 sg = R.segSmall[q];
		int gs = sg.x, n = sg.y - sg.x, z = sg.z;
		for ( int i = threadIdx.x; i < n; i += blockDim.x )
		{
			sIdx[i] = R.gIdx[gs + i];
			sCen[i] = R.gCen[gs + i];
			if ( i < n - 1 )
				sFreed[i] = R.freed[F - 1 - ( gs + z + i )];
		}
		if ( threadIdx.x == 0 )
		{
			sItem[0][0] = make_int4( 0, n, z, 0 );
			sCount[0] = 1;
			sCount[1] = 0;
			sm.kidCount = 0;
		}
		__syncthreads();
		int levels = 0;
		for ( int level = 0; level < PT_SMALL_LEVELS; ++level )
		{
			int cur = level & 1;
			int m = sCount[cur];
			if ( m == 0 )
				break;
			if ( threadIdx.x == 0 )
				sm.levelStart[level] = sm.kidCount;
			levels = level + 1;
			// items of at most PT_SERIAL nodes: a thread each
			for ( int it = threadIdx.x; it < m; it += blockDim.x )
			{
				int4 item = sItem[cur][it];
				if ( item.y - item.x <= PT_SERIAL )
					sSplit[it] = pt_partition_serial( sIdx, sCen, item.x, item.y );
			}
			// larger items: a warp each
			for ( int it = wid; it < m; it += PT_WARPS )
			{
				int4 item = sItem[cur][it];
				int s = item.x, e = item.y, cnt = e - s;
				if ( cnt <= PT_SERIAL )
					continue;
				int split = 1;
				{
					float lx = FLT_MAX, ly = FLT_MAX, hx = -FLT_MAX, hy = -FLT_MAX;
					for ( int i = s + lane; i < e; i += 32 )
					{
						float2 c = sCen[i];
						lx = c.x < lx ? c.x : lx;
						ly = c.y < ly ? c.y : ly;
						hx = c.x > hx ? c.x : hx;
						hy = c.y > hy ? c.y : hy;
					}
#pragma unroll
					for ( int o = 16; o > 0; o >>= 1 )
					{
						float v;
						v = __shfl_xor_sync( 0xffffffffu, lx, o );
						lx = v < lx ? v : lx;
						v = __shfl_xor_sync( 0xffffffffu, ly, o );
						ly = v < ly ? v : ly;
						v = __shfl_xor_sync( 0xffffffffu, hx, o );
						hx = v > hx ? v : hx;
						v = __shfl_xor_sync( 0xffffffffu, hy, o );
						hy = v > hy ? v : hy;
					}
					float dx = hx - lx, dy = hy - ly;
					bool axisY = !( dx > dy );
					float pivot = axisY ? 0.5f * ( ly + hy ) : 0.5f * ( lx + hx );
					int below = 0;
					for ( int base = s; base < e; base += 32 )
					{
						int i = base + lane;
						bool b = i < e && pt_axis( sCen[i], axisY ) < pivot;
						below += __popc( __ballot_sync( 0xffffffffu, b ) );
					}
					split = ( below == 0 || below == cnt ) ? cnt / 2 : below;
					if ( below != 0 && below != cnt )
					{
						int mid = s + below, run = 0, runR = 0;
						for ( int base = s; base < mid; base += 32 )
						{
							int i = base + lane;
							bool f = i < mid && !( pt_axis( sCen[i], axisY ) < pivot );
							unsigned mk = __ballot_sync( 0xffffffffu, f );
							if ( f )
								sBL[s + run + __popc( mk & lt )] = i;
							run += __popc( mk );
						}
						for ( int base = e - 1; base >= mid; base -= 32 )
						{
							int i = base - lane;
							bool f = i >= mid && pt_axis( sCen[i], axisY ) < pivot;
							unsigned mk = __ballot_sync( 0xffffffffu, f );
							if ( f )
								sBR[s + runR + __popc( mk & lt )] = i;
							runR += __popc( mk );
						}
						__syncwarp();
						for ( int k = lane; k < run; k += 32 )
						{
							int a = sBL[s + k], b = sBR[s + k];
							int ti = sIdx[a];
							sIdx[a] = sIdx[b];
							sIdx[b] = ti;
							float2 tc = sCen[a];
							sCen[a] = sCen[b];
							sCen[b] = tc;
						}
						__syncwarp();
					}
				}
				if ( lane == 0 )
					sSplit[it] = split;
			}
			__syncthreads();
			// link the level's nodes, queue the parts of two or more
			for ( int it = threadIdx.x; it < m; it += blockDim.x )
			{
				int4 item = sItem[cur][it];
				int s = item.x, e = item.y, c1 = item.z;
				int le = s + sSplit[it];
				int kn = s + c1 - z, kl = s + c1 + 1 - z, kr = le + c1 - z;
				if ( kn < 0 || kn >= n - 1 || ( le - s > 1 && ( kl < 0 || kl >= n - 1 ) ) ||
					 ( e - le > 1 && ( kr < 0 || kr >= n - 1 ) ) || le <= s || le >= e )
				{
					atomicOr( &sc->error, ERR_TREE );
					continue;
				}
				int node = sFreed[kn];
				int left = le - s == 1 ? sIdx[s] : sFreed[kl];
				int right = e - le == 1 ? sIdx[le] : sFreed[kr];
				T.child1[node] = left;
				T.child2[node] = right;
				T.parent[left] = node;
				T.parent[right] = node;
				// children by local slot: a gathered node by its position,
				// a new internal node by PT_SMALL + its freed position
				sm.kid[atomicAdd( &sm.kidCount, 1 )] =
					make_int4( kn, le - s == 1 ? s : PT_SMALL + kl, e - le == 1 ? le : PT_SMALL + kr, 0 );
				if ( le - s >= 2 )
					sItem[cur ^ 1][atomicAdd( &sCount[cur ^ 1], 1 )] = make_int4( s, le, c1 + 1, 0 );
				if ( e - le >= 2 )
					sItem[cur ^ 1][atomicAdd( &sCount[cur ^ 1], 1 )] = make_int4( le, e, c1, 0 );
			}
			__syncthreads();
			if ( threadIdx.x == 0 )
				sCount[cur] = 0;
			__syncthreads();
		}
		if ( threadIdx.x == 0 )
			sm.levelStart[levels] = sm.kidCount;
		__syncthreads();
		// boxes, heights, categories and leaf counts bottom up, a level at a
		// time in shared memory (dynamic_tree.c:1990-2010), each new node
		// written out once; the gathered nodes' values are read first
		for ( int i = threadIdx.x; i < n; i += blockDim.x )
		{
			int g = sIdx[i];
			sm.u.r.box[i] = T.box[g];
			sm.u.r.cat[i] = T.cat[g];
			sm.u.r.hl[i] = make_int2( T.height[g], T.leaves[g] );
		}
		__syncthreads();
		for ( int level = levels - 1; level >= 0; --level )
		{
			int k0 = sm.levelStart[level], k1 = sm.levelStart[level + 1];
			for ( int k = k0 + threadIdx.x; k < k1; k += blockDim.x )
			{
				int4 kd = sm.kid[k];
				float4 bx = pt_union( sm.u.r.box[kd.y], sm.u.r.box[kd.z] );
				unsigned long long ct = sm.u.r.cat[kd.y] | sm.u.r.cat[kd.z];
				int2 ha = sm.u.r.hl[kd.y], hb = sm.u.r.hl[kd.z];
				int2 hl = make_int2( 1 + max( ha.x, hb.x ), ha.y + hb.y );
				int slot = PT_SMALL + kd.x;
				sm.u.r.box[slot] = bx;
				sm.u.r.cat[slot] = ct;
				sm.u.r.hl[slot] = hl;
				int node = sFreed[kd.x];
				T.box[node] = bx;
				T.cat[node] = ct;
				T.height[node] = hl.x;
				T.leaves[node] = hl.y;
				T.flags[node] = PT_ALLOCATED;
			}
			__syncthreads();
		}
	}
}

// boxes, categories, heights and leaf counts of the large levels' new
// internal nodes, bottom up (the second child to arrive computes its parent)
__global__ void k_pt_refresh( DWorld w, int t )
{
	if ( w.sc->rbActive == 0 )
		return;
	const DProxyTree T = w.pt[t];
	const DRebuild R = w.rb;
	int n = w.sc->rbCount;
	int root = R.freed[n - 2];
	if ( blockIdx.x == 0 && threadIdx.x == 0 )
	{
		T.parent[root] = -1;
		w.sc->treeRoot[t] = root;
	}
	// the large levels' nodes only: k_pt_small did the nodes below them
	int starts = w.sc->rbRefresh;
	for ( int i = blockIdx.x * blockDim.x + threadIdx.x; i < starts; i += gridDim.x * blockDim.x )
	{
		int c = R.rfStart[i];
		for ( int guard = 0;; ++guard )
		{
			if ( guard > PT_GUARD )
			{
				atomicOr( &w.sc->error, ERR_TREE );
				break;
			}
			int p = T.parent[c];
			if ( p < 0 || p >= T.cap )
			{
				atomicOr( &w.sc->error, ERR_TREE );
				break;
			}
			if ( pt_atom_add( R.cnt + p, 1 ) == 0 )
				break;
			pt_refresh_node( T, p, T.child1[p], T.child2[p] );
			__threadfence();
			if ( p == root )
				break;
			c = p;
		}
	}
}

// left-to-right rank of every leaf and its inverse
__global__ void k_pt_ranks( DWorld w, int t, int onlyAfterRebuild )
{
	if ( onlyAfterRebuild && w.sc->rbActive == 0 )
		return;
	const DProxyTree T = w.pt[t];
	for ( int i = blockIdx.x * blockDim.x + threadIdx.x; i < T.cap; i += gridDim.x * blockDim.x )
	{
		if ( ( T.flags[i] & ( PT_ALLOCATED | PT_LEAF ) ) != ( PT_ALLOCATED | PT_LEAF ) )
			continue;
		int r = 0, c = i;
		for ( int guard = 0;; ++guard )
		{
			if ( guard > PT_GUARD )
			{
				atomicOr( &w.sc->error, ERR_TREE );
				break;
			}
			int p = T.parent[c];
			if ( p < 0 || p >= T.cap )
				break;
			if ( T.child2[p] == c )
				r += T.leaves[T.child1[p]];
			c = p;
		}
		T.rank[i] = r;
		if ( r >= 0 && r < T.cap )
			T.rankShape[r] = T.shape[i];
		else
			atomicOr( &w.sc->error, ERR_TREE );
	}
}

// ---------------------------------------------------------------------------
// host drivers
// ---------------------------------------------------------------------------
int pt_large_blocks()
{
	cudaFuncSetAttribute( k_pt_small, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof( PtSmall ) );
	cudaFuncSetAttribute( k_pt_large, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof( PtLarge ) );
	int perSM = 0;
	cudaOccupancyMaxActiveBlocksPerMultiprocessor( &perSM, k_pt_large, PT_THREADS, sizeof( PtLarge ) );
	int dev = 0, sms = 0;
	cudaGetDevice( &dev );
	cudaDeviceGetAttribute( &sms, cudaDevAttrMultiProcessorCount, dev );
	if ( perSM < 1 )
		return 0;
	return sms * ( perSM < 2 ? perSM : 2 );
}

// step start: the host's buffered proxies join the move array
void launch_pt_host_moves( DWorld& w, StepScratch& s, cudaStream_t st )
{
	k_pt_host_flags<<<grid_for( w.shapeCap ), 256, 0, st>>>( w, s.tmpA );
	scan_lookback( s.tmpA, s.tmpB, &w.sc->hostMoveCount, 0, w.shapeCap, nullptr, s.scanState, &w.sc->error, st );
	k_pt_host_write<<<grid_for( w.shapeCap ), 256, 0, st>>>( w, s.tmpA, s.tmpB );
	k_pt_host_done<<<1, 1, 0, st>>>( w, s.tmpA, s.tmpB );
}

void launch_pt_decode( DWorld& w, cudaStream_t st )
{
	k_pt_decode<<<grid_for( w.pairCap ), 256, 0, st>>>( w );
}

// collide phase: partial rebuild of the dynamic and kinematic trees
// (broad_phase.c:488-492)
void launch_pt_rebuild( DWorld& w, StepScratch& s, cudaStream_t st )
{
	for ( int t = 2; t >= 1; --t )
	{
		const DProxyTree& T = w.pt[t];
		if ( T.cap == 0 || w.ptProxies[t] == 0 )
			continue;
		int g = grid_for( T.cap );
		k_pt_mark<<<g, 256, 0, st>>>( w, t );
		k_pt_count<<<g, 256, 0, st>>>( w, t );
		k_pt_gather<<<g, 256, 0, st>>>( w, t );
		if ( s.ptBlocks > 0 )
		{
			unsigned* counter = &w.sc->ptBarrier;
			cudaMemsetAsync( counter, 0, sizeof( unsigned ), st );
			void* args[] = { &w, &t, &counter };
			cudaLaunchCooperativeKernel( (void*)k_pt_large, dim3( s.ptBlocks ), dim3( PT_THREADS ), args,
										 sizeof( PtLarge ), st );
		}
		k_pt_small<<<F2D_SMS * 2, PT_THREADS, sizeof( PtSmall ), st>>>( w, t );
		k_pt_refresh<<<g, 256, 0, st>>>( w, t );
	}
}

// finalize: the move array in awake order, proxies enlarged
void launch_pt_moves( DWorld& w, StepScratch& s, cudaStream_t st )
{
	int* count = w.isl ? (int*)( (char*)w.isl + offsetof( DIslands, awakeBodyCount ) ) : &w.sc->awakeOrderCount;
	k_pt_move_count<<<grid_for( w.bodyCap ), 256, 0, st>>>( w, s.tmpA );
	scan_lookback( s.tmpA, s.tmpB, count, w.bodyCount, w.bodyCap, &w.sc->moveArrayCount, s.scanState, &w.sc->error, st );
	k_pt_move_assign<<<grid_for( w.bodyCap ), 256, 0, st>>>( w, s.tmpB );
}

// after a host upload of tree t
void launch_pt_ranks( DWorld& w, cudaStream_t st, int t )
{
	if ( w.pt[t].cap > 0 )
		k_pt_ranks<<<grid_for( w.pt[t].cap ), 256, 0, st>>>( w, t, 0 );
}
