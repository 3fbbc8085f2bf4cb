/* tree_oracle.c -- plain-typed wrappers over the oracle's dynamic tree
 * (oracle/b2o_tree.c) for tree_check.c. */
#include "b2o.h"

#include <stdlib.h>

static oBox box_of( const float* b ) { return (oBox){ { b[0], b[1] }, { b[2], b[3] } }; }

void* ot_new( void )
{
	oTree* t = (oTree*)calloc( 1, sizeof( oTree ) );
	otree_init( t );
	return t;
}
void ot_free( void* t )
{
	otree_free( (oTree*)t );
	free( t );
}
int ot_create( void* t, const float* b, int user ) { return otree_create_proxy( (oTree*)t, box_of( b ), 1u, user ); }
void ot_destroy( void* t, int id ) { otree_destroy_proxy( (oTree*)t, id ); }
void ot_move( void* t, int id, const float* b ) { otree_move_proxy( (oTree*)t, id, box_of( b ) ); }
void ot_enlarge( void* t, int id, const float* b ) { otree_enlarge_proxy( (oTree*)t, id, box_of( b ) ); }
void ot_rebuild( void* t ) { otree_rebuild( (oTree*)t ); }

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

int ot_query( void* t, const float* b, int* out, int cap )
{
	Hits h = { out, 0, cap };
	otree_query( (oTree*)t, box_of( b ), 0xFFFFFFFFu, hit, &h );
	return h.n;
}

/* root, node count, then per node slot: box (as float bits), category, parent, child1,
 * child2, userData, height; a free slot only its free-list link and height */
int ot_dump( void* t, int* out, int cap )
{
	oTree* g = (oTree*)t;
	int n = 0;
	if ( n + 2 <= cap )
	{
		out[0] = g->root;
		out[1] = g->nodeCount;
	}
	n = 2;
	for ( int i = 0; i < g->capacity; ++i )
	{
		const oNode* d = g->nodes + i;
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
