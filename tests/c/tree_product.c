/* tree_product.c -- plain-typed wrappers over the library's host dynamic tree
 * (box2c_gb300/csrc/tree.c) for tree_check.c. */
#include "host.h"

#include <stdlib.h>

static b2gBox box_of( const float* b ) { return (b2gBox){ { b[0], b[1] }, { b[2], b[3] } }; }

void* pt_new( void )
{
	gTree* t = (gTree*)calloc( 1, sizeof( gTree ) );
	gtree_init( t );
	return t;
}
void pt_free( void* t )
{
	gtree_free( (gTree*)t );
	free( t );
}
int pt_create( void* t, const float* b, int user ) { return gtree_create_proxy( (gTree*)t, box_of( b ), 1u, user ); }
void pt_destroy( void* t, int id ) { gtree_destroy_proxy( (gTree*)t, id ); }
void pt_move( void* t, int id, const float* b ) { gtree_move_proxy( (gTree*)t, id, box_of( b ) ); }
void pt_enlarge( void* t, int id, const float* b ) { gtree_enlarge_proxy( (gTree*)t, id, box_of( b ) ); }
void pt_rebuild( void* t ) { gtree_rebuild( (gTree*)t ); }

typedef struct Hits
{
	int* out;
	int n, cap;
} Hits;

static bool hit( int proxyId, int userData, void* ctx )
{
	Hits* h = (Hits*)ctx;
	if ( h->n + 2 <= h->cap )
	{
		h->out[h->n] = proxyId;
		h->out[h->n + 1] = userData;
	}
	h->n += 2;
	return true;
}

int pt_query( void* t, const float* b, int* out, int cap )
{
	Hits h = { out, 0, cap };
	gtree_query( (gTree*)t, box_of( b ), 0xFFFFFFFFu, hit, &h );
	return h.n;
}

/* root, node count, then per node slot: box (as float bits), category, parent, child1,
 * child2, userData, height; a free slot only its free-list link and height */
int pt_dump( void* t, int* out, int cap )
{
	gTree* g = (gTree*)t;
	int n = 0;
	if ( n + 2 <= cap )
	{
		out[0] = g->root;
		out[1] = g->nodeCount;
	}
	n = 2;
	for ( int i = 0; i < g->capacity; ++i )
	{
		const gNode* d = g->nodes + i;
		int v[10];
		const float* f = &d->box.lo.x;
		for ( int k = 0; k < 4; ++k )
			v[k] = ( (const int*)f )[k];
		v[4] = (int)d->category;
		v[5] = d->parent;
		v[6] = d->child1;
		v[7] = d->child2;
		v[8] = d->userData;
		v[9] = d->height;
		if ( d->height < 0 )
		{
			/* a free slot: only the free-list link (next allocation order) counts */
			for ( int k = 0; k < 10; ++k )
				v[k] = k == 5 ? d->parent : k == 9 ? d->height : 0;
		}
		for ( int k = 0; k < 10; ++k, ++n )
			if ( n < cap )
				out[n] = v[k];
	}
	return n;
}
