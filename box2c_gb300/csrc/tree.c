/*
 * tree.c -- host dynamic AABB tree of the broadphase (three per world: static,
 * kinematic, dynamic).  Serial and order-sensitive, so it stays on the host: proxy ids
 * fix the A/B order and creation order of new contacts, which fix contact ids and
 * colours.
 *
 * Restates the reference src/dynamic_tree.c: node pool with LIFO free list (:78-124),
 * greedy surface-area sibling search (:142-294), rotations (:296-581), insert/remove
 * (:583-726), proxy create/move/enlarge (:728-823), depth-first query (:1120-1159) and
 * the partial rebuild with median split (:1363-1487, :1656-1925).  Node indices are
 * proxy ids and fix the A/B order of new pairs, so allocation order is reproduced.
 */
#include "host.h"

#include <string.h>

#define TREE_STACK 1024

void gtree_init( gTree* t )
{
	memset( t, 0, sizeof( *t ) );
	t->root = B2G_NULL;
	t->freeList = B2G_NULL;
	t->nodes = (gNode*)b2g_calloc( 16, sizeof( gNode ) );
	if ( t->nodes == NULL )
		return;
	t->capacity = 16;
	t->reserved = 16;
	for ( int i = 0; i < t->capacity - 1; ++i )
	{
		t->nodes[i].parent = i + 1;
		t->nodes[i].height = -1;
	}
	t->nodes[t->capacity - 1].parent = B2G_NULL;
	t->nodes[t->capacity - 1].height = -1;
	t->freeList = 0;
}

void gtree_free( gTree* t )
{
	b2g_free( t->nodes );
	b2g_free( t->leafIndices );
	b2g_free( t->leafCenters );
	memset( t, 0, sizeof( *t ) );
}

/* Capacity after the next growth: by half, as the reference grows its pool, so that
 * node indices follow its allocation order. */
static int next_capacity( int cap ) { return cap < 16 ? 16 : cap + ( cap >> 1 ); }

/* Makes the allocation hold `count` nodes without changing the pool.  False when
 * memory ran out. */
static bool reserve_nodes( gTree* t, int count )
{
	if ( count <= t->reserved )
		return true;
	gNode* nodes = (gNode*)b2g_realloc( t->nodes, sizeof( gNode ) * (size_t)count );
	if ( nodes == NULL )
		return false;
	t->nodes = nodes;
	t->reserved = count;
	return true;
}

/* Grows the pool when the free list is empty.  False when memory ran out. */
static bool grow_nodes( gTree* t )
{
	if ( t->freeList != B2G_NULL )
		return true;
	int cap = next_capacity( t->capacity );
	if ( reserve_nodes( t, cap ) == false )
		return false;
	t->capacity = cap;
	for ( int i = t->nodeCount; i < t->capacity - 1; ++i )
	{
		t->nodes[i].parent = i + 1;
		t->nodes[i].height = -1;
	}
	t->nodes[t->capacity - 1].parent = B2G_NULL;
	t->nodes[t->capacity - 1].height = -1;
	t->freeList = t->nodeCount;
	return true;
}

static int alloc_node( gTree* t )
{
	grow_nodes( t );
	int id = t->freeList;
	gNode* n = t->nodes + id;
	t->freeList = n->parent;
	memset( n, 0, sizeof( *n ) );
	n->parent = B2G_NULL;
	n->child1 = B2G_NULL;
	n->child2 = B2G_NULL;
	n->userData = -1;
	n->height = -2;
	t->nodeCount += 1;
	return id;
}

static void free_node( gTree* t, int id )
{
	t->nodes[id].parent = t->freeList;
	t->nodes[id].height = -1;
	t->freeList = id;
	t->nodeCount -= 1;
}

static int16_t max16( int16_t a, int16_t b ) { return a > b ? a : b; }

static int find_best_sibling( const gTree* t, b2gBox boxD )
{
	b2gVec centerD = gbox_center( boxD );
	float areaD = gbox_perimeter( boxD );
	const gNode* nodes = t->nodes;
	int root = t->root;
	b2gBox rootBox = nodes[root].box;
	float areaBase = gbox_perimeter( rootBox );
	float directCost = gbox_perimeter( gbox_union( rootBox, boxD ) );
	float inheritedCost = 0;
	int best = root;
	float bestCost = directCost;
	int index = root;
	while ( nodes[index].height > 0 )
	{
		int c1 = nodes[index].child1;
		int c2 = nodes[index].child2;
		float cost = directCost + inheritedCost;
		if ( cost < bestCost )
		{
			best = index;
			bestCost = cost;
		}
		inheritedCost += directCost - areaBase;

		bool leaf1 = nodes[c1].height == 0;
		bool leaf2 = nodes[c2].height == 0;

		float lower1 = FLT_MAX;
		b2gBox box1 = nodes[c1].box;
		float direct1 = gbox_perimeter( gbox_union( box1, boxD ) );
		float area1 = 0;
		if ( leaf1 )
		{
			float cost1 = direct1 + inheritedCost;
			if ( cost1 < bestCost )
			{
				best = c1;
				bestCost = cost1;
			}
		}
		else
		{
			area1 = gbox_perimeter( box1 );
			lower1 = inheritedCost + direct1 + gmin( areaD - area1, 0 );
		}

		float lower2 = FLT_MAX;
		b2gBox box2 = nodes[c2].box;
		float direct2 = gbox_perimeter( gbox_union( box2, boxD ) );
		float area2 = 0;
		if ( leaf2 )
		{
			float cost2 = direct2 + inheritedCost;
			if ( cost2 < bestCost )
			{
				best = c2;
				bestCost = cost2;
			}
		}
		else
		{
			area2 = gbox_perimeter( box2 );
			lower2 = inheritedCost + direct2 + gmin( areaD - area2, 0 );
		}

		if ( leaf1 && leaf2 )
			break;
		if ( bestCost <= lower1 && bestCost <= lower2 )
			break;
		if ( lower1 == lower2 && leaf1 == false )
		{
			b2gVec d1 = gsub( gbox_center( box1 ), centerD );
			b2gVec d2 = gsub( gbox_center( box2 ), centerD );
			lower1 = glen2( d1 );
			lower2 = glen2( d2 );
		}
		if ( lower1 < lower2 && leaf1 == false )
		{
			index = c1;
			areaBase = area1;
			directCost = direct1;
		}
		else
		{
			index = c2;
			areaBase = area2;
			directCost = direct2;
		}
	}
	return best;
}

/* Re-derives node X's summary from its two children (box given explicitly). */
static void set_parent( gNode* X, b2gBox box, const gNode* a, const gNode* b )
{
	X->box = box;
	X->height = 1 + max16( a->height, b->height );
	X->category = a->category | b->category;
	X->enlarged = a->enlarged || b->enlarged;
}

static void rotate_nodes( gTree* t, int iA )
{
	gNode* nodes = t->nodes;
	gNode* A = nodes + iA;
	if ( A->height < 2 )
		return;
	int iB = A->child1, iC = A->child2;
	gNode* B = nodes + iB;
	gNode* C = nodes + iC;

	if ( B->height == 0 )
	{
		/* B leaf, C internal: try swapping B with a child of C */
		int iF = C->child1, iG = C->child2;
		gNode* F = nodes + iF;
		gNode* G = nodes + iG;
		float costBase = gbox_perimeter( C->box );
		b2gBox boxBG = gbox_union( B->box, G->box );
		float costBF = gbox_perimeter( boxBG );
		b2gBox boxBF = gbox_union( B->box, F->box );
		float costBG = gbox_perimeter( boxBF );
		if ( costBase < costBF && costBase < costBG )
			return;
		if ( costBF < costBG )
		{
			A->child1 = iF;
			C->child1 = iB;
			B->parent = iC;
			F->parent = iA;
			set_parent( C, boxBG, B, G );
			A->height = 1 + max16( C->height, F->height );
			A->category = C->category | F->category;
			A->enlarged = C->enlarged || F->enlarged;
		}
		else
		{
			A->child1 = iG;
			C->child2 = iB;
			B->parent = iC;
			G->parent = iA;
			set_parent( C, boxBF, B, F );
			A->height = 1 + max16( C->height, G->height );
			A->category = C->category | G->category;
			A->enlarged = C->enlarged || G->enlarged;
		}
	}
	else if ( C->height == 0 )
	{
		/* C leaf, B internal: try swapping C with a child of B */
		int iD = B->child1, iE = B->child2;
		gNode* D = nodes + iD;
		gNode* E = nodes + iE;
		float costBase = gbox_perimeter( B->box );
		b2gBox boxCE = gbox_union( C->box, E->box );
		float costCD = gbox_perimeter( boxCE );
		b2gBox boxCD = gbox_union( C->box, D->box );
		float costCE = gbox_perimeter( boxCD );
		if ( costBase < costCD && costBase < costCE )
			return;
		if ( costCD < costCE )
		{
			A->child2 = iD;
			B->child1 = iC;
			C->parent = iB;
			D->parent = iA;
			set_parent( B, boxCE, C, E );
			A->height = 1 + max16( B->height, D->height );
			A->category = B->category | D->category;
			A->enlarged = B->enlarged || D->enlarged;
		}
		else
		{
			A->child2 = iE;
			B->child2 = iC;
			C->parent = iB;
			E->parent = iA;
			set_parent( B, boxCD, C, D );
			A->height = 1 + max16( B->height, E->height );
			A->category = B->category | E->category;
			A->enlarged = B->enlarged || E->enlarged;
		}
	}
	else
	{
		int iD = B->child1, iE = B->child2, iF = C->child1, iG = C->child2;
		gNode* D = nodes + iD;
		gNode* E = nodes + iE;
		gNode* F = nodes + iF;
		gNode* G = nodes + iG;
		float areaB = gbox_perimeter( B->box );
		float areaC = gbox_perimeter( C->box );
		float bestCost = areaB + areaC;
		int best = 0; /* 0 none, 1 BF, 2 BG, 3 CD, 4 CE */
		b2gBox boxBG = gbox_union( B->box, G->box );
		float costBF = areaB + gbox_perimeter( boxBG );
		if ( costBF < bestCost )
		{
			best = 1;
			bestCost = costBF;
		}
		b2gBox boxBF = gbox_union( B->box, F->box );
		float costBG = areaB + gbox_perimeter( boxBF );
		if ( costBG < bestCost )
		{
			best = 2;
			bestCost = costBG;
		}
		b2gBox boxCE = gbox_union( C->box, E->box );
		float costCD = areaC + gbox_perimeter( boxCE );
		if ( costCD < bestCost )
		{
			best = 3;
			bestCost = costCD;
		}
		b2gBox boxCD = gbox_union( C->box, D->box );
		float costCE = areaC + gbox_perimeter( boxCD );
		if ( costCE < bestCost )
			best = 4;

		switch ( best )
		{
			case 1:
				A->child1 = iF;
				C->child1 = iB;
				B->parent = iC;
				F->parent = iA;
				set_parent( C, boxBG, B, G );
				A->height = 1 + max16( C->height, F->height );
				A->category = C->category | F->category;
				A->enlarged = C->enlarged || F->enlarged;
				break;
			case 2:
				A->child1 = iG;
				C->child2 = iB;
				B->parent = iC;
				G->parent = iA;
				set_parent( C, boxBF, B, F );
				A->height = 1 + max16( C->height, G->height );
				A->category = C->category | G->category;
				A->enlarged = C->enlarged || G->enlarged;
				break;
			case 3:
				A->child2 = iD;
				B->child1 = iC;
				C->parent = iB;
				D->parent = iA;
				set_parent( B, boxCE, C, E );
				A->height = 1 + max16( B->height, D->height );
				A->category = B->category | D->category;
				A->enlarged = B->enlarged || D->enlarged;
				break;
			case 4:
				A->child2 = iE;
				B->child2 = iC;
				C->parent = iB;
				E->parent = iA;
				set_parent( B, boxCD, C, D );
				A->height = 1 + max16( B->height, E->height );
				A->category = B->category | E->category;
				A->enlarged = B->enlarged || E->enlarged;
				break;
			default:
				break;
		}
	}
}

static void insert_leaf( gTree* t, int leaf, bool shouldRotate )
{
	if ( t->root == B2G_NULL )
	{
		t->root = leaf;
		t->nodes[leaf].parent = B2G_NULL;
		return;
	}
	b2gBox leafBox = t->nodes[leaf].box;
	int sibling = find_best_sibling( t, leafBox );
	int oldParent = t->nodes[sibling].parent;
	int newParent = alloc_node( t );
	gNode* nodes = t->nodes;
	nodes[newParent].parent = oldParent;
	nodes[newParent].userData = -1;
	nodes[newParent].box = gbox_union( leafBox, nodes[sibling].box );
	nodes[newParent].category = nodes[leaf].category | nodes[sibling].category;
	nodes[newParent].height = nodes[sibling].height + 1;
	if ( oldParent != B2G_NULL )
	{
		if ( nodes[oldParent].child1 == sibling )
			nodes[oldParent].child1 = newParent;
		else
			nodes[oldParent].child2 = newParent;
	}
	else
	{
		t->root = newParent;
	}
	nodes[newParent].child1 = sibling;
	nodes[newParent].child2 = leaf;
	nodes[sibling].parent = newParent;
	nodes[leaf].parent = newParent;

	int index = nodes[leaf].parent;
	while ( index != B2G_NULL )
	{
		int c1 = nodes[index].child1;
		int c2 = nodes[index].child2;
		set_parent( nodes + index, gbox_union( nodes[c1].box, nodes[c2].box ), nodes + c1, nodes + c2 );
		if ( shouldRotate )
			rotate_nodes( t, index );
		index = nodes[index].parent;
	}
}

static void remove_leaf( gTree* t, int leaf )
{
	if ( leaf == t->root )
	{
		t->root = B2G_NULL;
		return;
	}
	gNode* nodes = t->nodes;
	int parent = nodes[leaf].parent;
	int grand = nodes[parent].parent;
	int sibling = nodes[parent].child1 == leaf ? nodes[parent].child2 : nodes[parent].child1;
	if ( grand != B2G_NULL )
	{
		if ( nodes[grand].child1 == parent )
			nodes[grand].child1 = sibling;
		else
			nodes[grand].child2 = sibling;
		nodes[sibling].parent = grand;
		free_node( t, parent );
		int index = grand;
		while ( index != B2G_NULL )
		{
			gNode* n = nodes + index;
			gNode* a = nodes + n->child1;
			gNode* b = nodes + n->child2;
			/* the reference leaves the enlarged flag untouched here */
			n->box = gbox_union( a->box, b->box );
			n->category = a->category | b->category;
			n->height = 1 + max16( a->height, b->height );
			index = n->parent;
		}
	}
	else
	{
		t->root = sibling;
		nodes[sibling].parent = B2G_NULL;
		free_node( t, parent );
	}
}

int gtree_create_proxy( gTree* t, b2gBox box, uint32_t category, int userData )
{
	/* a leaf and, on insertion, a new parent: the memory of a pool growth is held before
	 * the tree changes, so the insertion cannot fail half way */
	bool twoFree = t->freeList != B2G_NULL && t->nodes[t->freeList].parent != B2G_NULL;
	if ( twoFree == false && reserve_nodes( t, next_capacity( t->capacity ) ) == false )
		return B2G_NULL;
	int id = alloc_node( t );
	gNode* n = t->nodes + id;
	n->box = box;
	n->userData = userData;
	n->category = category;
	n->height = 0;
	insert_leaf( t, id, true );
	t->proxyCount += 1;
	return id;
}

void gtree_destroy_proxy( gTree* t, int proxyId )
{
	remove_leaf( t, proxyId );
	free_node( t, proxyId );
	t->proxyCount -= 1;
}

void gtree_move_proxy( gTree* t, int proxyId, b2gBox box )
{
	remove_leaf( t, proxyId );
	t->nodes[proxyId].box = box;
	insert_leaf( t, proxyId, false );
}

void gtree_enlarge_proxy( gTree* t, int proxyId, b2gBox box )
{
	gNode* nodes = t->nodes;
	nodes[proxyId].box = box;
	int p = nodes[proxyId].parent;
	while ( p != B2G_NULL )
	{
		bool changed = gbox_enlarge( &nodes[p].box, box );
		nodes[p].enlarged = true;
		p = nodes[p].parent;
		if ( changed == false )
			break;
	}
	while ( p != B2G_NULL )
	{
		if ( nodes[p].enlarged )
			break;
		nodes[p].enlarged = true;
		p = nodes[p].parent;
	}
}

int gtree_height( const gTree* t )
{
	return t->root == B2G_NULL ? 0 : t->nodes[t->root].height;
}

void gtree_query( const gTree* t, b2gBox box, uint32_t mask, gQueryFcn* fcn, void* ctx )
{
	int stack[TREE_STACK];
	int n = 0;
	stack[n++] = t->root;
	while ( n > 0 )
	{
		int id = stack[--n];
		if ( id == B2G_NULL )
			continue;
		const gNode* node = t->nodes + id;
		if ( gbox_overlaps( node->box, box ) && ( node->category & mask ) != 0 )
		{
			if ( node->height == 0 )
			{
				if ( fcn( id, node->userData, ctx ) == false )
					return;
			}
			else if ( n < TREE_STACK - 1 )
			{
				stack[n++] = node->child1;
				stack[n++] = node->child2;
			}
		}
	}
}

/* Median split on the longest axis of the leaf centres (Hoare partition). */
static int partition_mid( int* idx, b2gVec* c, int count )
{
	if ( count <= 2 )
		return count / 2;
	b2gVec lo = c[0], hi = c[0];
	for ( int i = 1; i < count; ++i )
	{
		lo = gminv( lo, c[i] );
		hi = gmaxv( hi, c[i] );
	}
	b2gVec d = gsub( hi, lo );
	b2gVec mid = gv( 0.5f * ( lo.x + hi.x ), 0.5f * ( lo.y + hi.y ) );
	int i1 = 0, i2 = count;
	bool useX = d.x > d.y;
	float pivot = useX ? mid.x : mid.y;
	while ( i1 < i2 )
	{
		while ( i1 < i2 && ( useX ? c[i1].x : c[i1].y ) < pivot )
			i1 += 1;
		while ( i1 < i2 && ( useX ? c[i2 - 1].x : c[i2 - 1].y ) >= pivot )
			i2 -= 1;
		if ( i1 < i2 )
		{
			int ti = idx[i1];
			idx[i1] = idx[i2 - 1];
			idx[i2 - 1] = ti;
			b2gVec tc = c[i1];
			c[i1] = c[i2 - 1];
			c[i2 - 1] = tc;
			i1 += 1;
			i2 -= 1;
		}
	}
	if ( i1 > 0 && i1 < count )
		return i1;
	return count / 2;
}

typedef struct oBuildItem
{
	int nodeIndex, childCount, start, split, end;
} oBuildItem;

static int build_tree( gTree* t, int leafCount )
{
	int* leaves = t->leafIndices;
	b2gVec* centers = t->leafCenters;
	if ( leafCount == 1 )
	{
		t->nodes[leaves[0]].parent = B2G_NULL;
		return leaves[0];
	}
	oBuildItem stack[TREE_STACK];
	int top = 0;
	stack[0].nodeIndex = alloc_node( t );
	stack[0].childCount = -1;
	stack[0].start = 0;
	stack[0].end = leafCount;
	stack[0].split = partition_mid( leaves, centers, leafCount );

	for ( ;; )
	{
		oBuildItem* item = stack + top;
		item->childCount += 1;
		if ( item->childCount == 2 )
		{
			if ( top == 0 )
				break;
			oBuildItem* parentItem = stack + ( top - 1 );
			gNode* nodes = t->nodes;
			gNode* parentNode = nodes + parentItem->nodeIndex;
			if ( parentItem->childCount == 0 )
				parentNode->child1 = item->nodeIndex;
			else
				parentNode->child2 = item->nodeIndex;
			gNode* node = nodes + item->nodeIndex;
			node->parent = parentItem->nodeIndex;
			gNode* a = nodes + node->child1;
			gNode* b = nodes + node->child2;
			node->box = gbox_union( a->box, b->box );
			node->height = 1 + max16( a->height, b->height );
			node->category = a->category | b->category;
			top -= 1;
		}
		else
		{
			int s = item->childCount == 0 ? item->start : item->split;
			int e = item->childCount == 0 ? item->split : item->end;
			int count = e - s;
			if ( count == 1 )
			{
				int child = leaves[s];
				gNode* node = t->nodes + item->nodeIndex;
				if ( item->childCount == 0 )
					node->child1 = child;
				else
					node->child2 = child;
				t->nodes[child].parent = item->nodeIndex;
			}
			else
			{
				top += 1;
				oBuildItem* ni = stack + top;
				ni->nodeIndex = alloc_node( t );
				ni->childCount = -1;
				ni->start = s;
				ni->end = e;
				ni->split = partition_mid( leaves + s, centers + s, count ) + s;
			}
		}
	}
	gNode* nodes = t->nodes;
	gNode* root = nodes + stack[0].nodeIndex;
	gNode* a = nodes + root->child1;
	gNode* b = nodes + root->child2;
	root->box = gbox_union( a->box, b->box );
	root->height = 1 + max16( a->height, b->height );
	root->category = a->category | b->category;
	return stack[0].nodeIndex;
}

void gtree_rebuild( gTree* t )
{
	int proxyCount = t->proxyCount;
	if ( proxyCount == 0 )
		return;
	if ( proxyCount > t->rebuildCapacity )
	{
		int cap = proxyCount + proxyCount / 2;
		int* li = (int*)b2g_alloc( sizeof( int ) * (size_t)cap );
		b2gVec* lc = (b2gVec*)b2g_alloc( sizeof( b2gVec ) * (size_t)cap );
		if ( li == NULL || lc == NULL )
		{
			/* no room for the rebuild's scratch: the tree stays as it is, still valid */
			b2g_free( li );
			b2g_free( lc );
			return;
		}
		b2g_free( t->leafIndices );
		b2g_free( t->leafCenters );
		t->leafIndices = li;
		t->leafCenters = lc;
		t->rebuildCapacity = cap;
	}
	int leafCount = 0;
	int stack[TREE_STACK];
	int n = 0;
	int index = t->root;
	gNode* nodes = t->nodes;
	gNode* node = nodes + index;
	for ( ;; )
	{
		if ( node->height == 0 || node->enlarged == false )
		{
			t->leafIndices[leafCount] = index;
			t->leafCenters[leafCount] = gbox_center( node->box );
			leafCount += 1;
			node->parent = B2G_NULL;
		}
		else
		{
			int doomed = index;
			index = node->child1;
			if ( n < TREE_STACK )
				stack[n++] = node->child2;
			node = nodes + index;
			free_node( t, doomed );
			continue;
		}
		if ( n == 0 )
			break;
		index = stack[--n];
		node = nodes + index;
	}
	t->root = build_tree( t, leafCount );
}
