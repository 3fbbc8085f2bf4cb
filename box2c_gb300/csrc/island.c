/*
 * island.c -- persistent islands, solver sets and sleep on the host.
 *
 * Island bookkeeping is serial, pointer-chasing integer work over linked lists, so it
 * stays on the host with the rest of the order-sensitive records; the device learns the
 * outcome through three channels: body operations (a body stops or starts being
 * integrated, a woken body's velocity and sleep timer are zeroed), the awake body list,
 * and the set bit of each contact (sleeping contacts are skipped by the narrowphase).
 * The device's finalisation kernel reports which bodies are past the sleep time; the
 * island decisions are made here from that report.
 *
 * Follows the reference: src/island.c:16-865 (islands, union-find linking, merging the
 * awake islands at the start of the solve, splitting an island by depth-first search),
 * src/solver_set.c:16-554 (waking a set, putting an island to sleep, merging two sleeping
 * sets), src/body.c:84-159 and :325-333 (a body's own island, leaving an island, waking a
 * body) and src/solver.c:281-298, :1956-2001 (which islands stay awake, the split
 * candidate, sleeping in reverse island order).  The order in which bodies, contacts and
 * joints move between sets fixes the awake order, the colours and the ids of later
 * steps, so every loop keeps the reference's order.
 */
#include "host.h"

#include <string.h>

static bool grow_islands( gWorld* w, int need )
{
	if ( need <= w->islandCap )
		return true;
	int nc = w->islandCap < 16 ? 16 : w->islandCap;
	while ( nc < need )
		nc *= 2;
	gIsland* p = (gIsland*)b2g_realloc( w->islands, sizeof( gIsland ) * (size_t)nc );
	if ( p == NULL )
		return false;
	memset( p + w->islandCap, 0, sizeof( gIsland ) * (size_t)( nc - w->islandCap ) );
	w->islands = p;
	w->islandCap = nc;
	return true;
}

static bool grow_sets( gWorld* w, int need )
{
	if ( need <= w->setCap )
		return true;
	int nc = w->setCap < 8 ? 8 : w->setCap;
	while ( nc < need )
		nc *= 2;
	gSolverSet* p = (gSolverSet*)b2g_realloc( w->sets, sizeof( gSolverSet ) * (size_t)nc );
	if ( p == NULL )
		return false;
	memset( p + w->setCap, 0, sizeof( gSolverSet ) * (size_t)( nc - w->setCap ) );
	for ( int i = w->setCap; i < nc; ++i )
		p[i].setIndex = B2G_NULL;
	w->sets = p;
	w->setCap = nc;
	return true;
}

void gislands_init( gWorld* w )
{
	/* set ids 0, 1 and 2 are the static, disabled and awake sets (reference
	 * src/world.c:140-160) */
	for ( int i = 0; i < G_SET_FIRST_SLEEPING; ++i )
		gid_alloc( &w->setIds );
	grow_sets( w, G_SET_FIRST_SLEEPING );
	w->splitIslandId = B2G_NULL;
}

void gislands_free( gWorld* w )
{
	for ( int i = 0; i < w->setCap; ++i )
	{
		gia_free( &w->sets[i].bodies );
		gia_free( &w->sets[i].contacts );
		gia_free( &w->sets[i].joints );
		gia_free( &w->sets[i].islands );
	}
	b2g_free( w->sets );
	b2g_free( w->islands );
	b2g_free( w->bodyOpSlot );
	b2g_free( w->islandSleepy );
	gia_free( &w->islandIds.freeIds );
	gia_free( &w->setIds.freeIds );
	gia_free( &w->awakeIslands );
	gia_free( &w->disabledContacts );
	gia_free( &w->staticJoints );
	gia_free( &w->bodyOps );
}

/* The awake set's bodies are the awake list; static bodies keep no list. */
gIntArray* gsolver_set_bodies( gWorld* w, int setIndex ) { return setIndex == G_SET_AWAKE ? &w->awake : &w->sets[setIndex].bodies; }

gIntArray* gsolver_set_contacts( gWorld* w, int setIndex )
{
	if ( setIndex == G_SET_AWAKE )
		return &w->nonTouching;
	if ( setIndex == G_SET_DISABLED )
		return &w->disabledContacts;
	return &w->sets[setIndex].contacts;
}

gIntArray* gsolver_set_joints( gWorld* w, int setIndex )
{
	return setIndex == G_SET_STATIC ? &w->staticJoints : &w->sets[setIndex].joints;
}

static gIntArray* set_islands( gWorld* w, int setIndex )
{
	return setIndex == G_SET_AWAKE ? &w->awakeIslands : &w->sets[setIndex].islands;
}

void gbody_remove_from_set( gWorld* w, gBody* b )
{
	if ( b->setIndex == G_SET_STATIC )
		return;
	if ( b->setIndex == G_SET_AWAKE )
	{
		int at = b->awakeIndex;
		int moved = gia_remove_swap( &w->awake, at );
		if ( moved != B2G_NULL )
			w->bodies[w->awake.data[at]].awakeIndex = at;
		w->awakeDirty = true;
	}
	else
	{
		gIntArray* list = &w->sets[b->setIndex].bodies;
		int at = b->setLocal;
		int moved = gia_remove_swap( list, at );
		if ( moved != B2G_NULL )
			w->bodies[list->data[at]].setLocal = at;
	}
	b->awakeIndex = B2G_NULL;
	b->setLocal = B2G_NULL;
}

/* ------------------------------------------------------------ device staging */
static void stage_op( gWorld* w, int bodyId, int code, bool mirror )
{
	if ( bodyId >= w->bodyOpSlotCap )
	{
		int nc = w->bodyOpSlotCap < 64 ? 64 : w->bodyOpSlotCap;
		while ( nc <= bodyId )
			nc *= 2;
		int* p = (int*)b2g_realloc( w->bodyOpSlot, sizeof( int ) * (size_t)nc );
		if ( p == NULL )
			return;
		for ( int i = w->bodyOpSlotCap; i < nc; ++i )
			p[i] = B2G_NULL;
		w->bodyOpSlot = p;
		w->bodyOpSlotCap = nc;
	}
	int op = ( bodyId << 2 ) | code;
	int slot = w->bodyOpSlot[bodyId];
	if ( slot != B2G_NULL )
		w->bodyOps.data[slot] = op;
	else
	{
		w->bodyOpSlot[bodyId] = w->bodyOps.count;
		gia_push( &w->bodyOps, op );
	}
	/* the body info is the host's; the state mirror follows when it is current */
	if ( mirror == false )
		return;
	if ( code == B2G_BODY_WAKE )
	{
		w->hInfo[bodyId] |= B2G_B_AWAKE;
		if ( w->mirrorStale == false )
		{
			float* st = w->hState + 8 * bodyId;
			st[0] = st[1] = st[2] = 0.0f;
			st[4] = st[5] = 0.0f;
			st[6] = 1.0f;
			st[7] = 0.0f;
		}
	}
	else
		w->hInfo[bodyId] &= ~B2G_B_AWAKE;
}

void gbody_stage_op( gWorld* w, int bodyId, int code ) { stage_op( w, bodyId, code, true ); }

void gbody_stage_new( gWorld* w, int bodyId, int code ) { stage_op( w, bodyId, code, false ); }

int gbody_flush_ops( gWorld* w )
{
	int e = 0;
	if ( w->bodyOps.count > 0 || w->awakeDirty )
		e |= b2gd_reserve( &w->dev, &w->io, w->bodyIds.next, w->shapeIds.next, w->contactIds.next, w->jointIds.next,
						   w->contactIds.next, w->shapeIds.next );
	if ( w->bodyOps.count > 0 )
	{
		e |= b2gd_body_ops( &w->dev, w->bodyOps.data, w->bodyOps.count );
		for ( int i = 0; i < w->bodyOps.count; ++i )
			w->bodyOpSlot[w->bodyOps.data[i] >> 2] = B2G_NULL;
		w->bodyOps.count = 0;
	}
	if ( w->awakeDirty )
	{
		e |= b2gd_upload_awake( &w->dev, w->awake.data, w->awake.count );
		w->awakeDirty = false;
	}
	return e;
}

/* ------------------------------------------------------------ islands */
static gIsland* create_island( gWorld* w, int setIndex )
{
	int islandId = gid_alloc( &w->islandIds );
	if ( grow_islands( w, islandId + 1 ) == false )
	{
		gid_unalloc( &w->islandIds, islandId );
		return NULL;
	}
	gIntArray* list = set_islands( w, setIndex );
	gIsland* island = w->islands + islandId;
	island->setIndex = setIndex;
	island->localIndex = list->count;
	island->islandId = islandId;
	island->headBody = island->tailBody = B2G_NULL;
	island->bodyCount = 0;
	island->headContact = island->tailContact = B2G_NULL;
	island->contactCount = 0;
	island->headJoint = island->tailJoint = B2G_NULL;
	island->jointCount = 0;
	island->parentIsland = B2G_NULL;
	island->constraintRemoveCount = 0;
	gia_push( list, islandId );
	return island;
}

static void destroy_island( gWorld* w, int islandId )
{
	gIsland* island = w->islands + islandId;
	gIntArray* list = set_islands( w, island->setIndex );
	int moved = gia_remove_swap( list, island->localIndex );
	if ( moved != B2G_NULL )
		w->islands[list->data[island->localIndex]].localIndex = island->localIndex;
	island->islandId = B2G_NULL;
	island->setIndex = B2G_NULL;
	island->localIndex = B2G_NULL;
	gid_free( &w->islandIds, islandId );
}

void gisland_create_for_body( gWorld* w, int setIndex, gBody* b )
{
	gIsland* island = create_island( w, setIndex );
	if ( island == NULL )
		return;
	b->islandId = island->islandId;
	island->headBody = b->id;
	island->tailBody = b->id;
	island->bodyCount = 1;
}

void gisland_remove_body( gWorld* w, gBody* b )
{
	if ( b->islandId == B2G_NULL )
		return;
	gIsland* island = w->islands + b->islandId;
	if ( b->islandPrev != B2G_NULL )
		w->bodies[b->islandPrev].islandNext = b->islandNext;
	if ( b->islandNext != B2G_NULL )
		w->bodies[b->islandNext].islandPrev = b->islandPrev;
	island->bodyCount -= 1;
	if ( island->headBody == b->id )
	{
		island->headBody = b->islandNext;
		if ( island->headBody == B2G_NULL )
			destroy_island( w, island->islandId );
	}
	else if ( island->tailBody == b->id )
		island->tailBody = b->islandPrev;
	b->islandId = B2G_NULL;
	b->islandPrev = B2G_NULL;
	b->islandNext = B2G_NULL;
}

/* Follows parent links to the root, halving the path on the way. */
static int island_root( gWorld* w, int islandId )
{
	gIsland* island = w->islands + islandId;
	while ( island->parentIsland != B2G_NULL )
	{
		gIsland* parent = w->islands + island->parentIsland;
		if ( parent->parentIsland != B2G_NULL )
			island->parentIsland = parent->parentIsland;
		islandId = island->parentIsland;
		island = parent;
	}
	return islandId;
}

static void push_contact( gWorld* w, int islandId, gContact* c )
{
	gIsland* island = w->islands + islandId;
	if ( island->headContact != B2G_NULL )
	{
		c->islandNext = island->headContact;
		w->contacts[island->headContact].islandPrev = c->id;
	}
	island->headContact = c->id;
	if ( island->tailContact == B2G_NULL )
		island->tailContact = island->headContact;
	island->contactCount += 1;
	c->islandId = islandId;
}

static void push_joint( gWorld* w, int islandId, gJoint* j )
{
	gIsland* island = w->islands + islandId;
	if ( island->headJoint != B2G_NULL )
	{
		j->islandNext = island->headJoint;
		w->joints[island->headJoint].islandPrev = j->id;
	}
	island->headJoint = j->id;
	if ( island->tailJoint == B2G_NULL )
		island->tailJoint = island->headJoint;
	island->jointCount += 1;
	j->islandId = islandId;
}

/* Joins the roots of the two bodies' islands (the second under the first) and returns the
 * island the new constraint goes to.  The path halving of the reference's two loops
 * leaves the same parent links as island_root. */
static int link_islands( gWorld* w, int islandIdA, int islandIdB )
{
	int rootA = islandIdA != B2G_NULL ? island_root( w, islandIdA ) : B2G_NULL;
	int rootB = islandIdB != B2G_NULL ? island_root( w, islandIdB ) : B2G_NULL;
	if ( rootA != rootB && rootA != B2G_NULL && rootB != B2G_NULL )
		w->islands[rootB].parentIsland = rootA;
	return rootA != B2G_NULL ? rootA : rootB;
}

void gisland_link_contact( gWorld* w, gContact* c )
{
	gBody* bodyA = w->bodies + c->edges[0].bodyId;
	gBody* bodyB = w->bodies + c->edges[1].bodyId;
	if ( bodyA->setIndex == G_SET_AWAKE && bodyB->setIndex >= G_SET_FIRST_SLEEPING )
		gsolver_set_wake( w, bodyB->setIndex );
	if ( bodyB->setIndex == G_SET_AWAKE && bodyA->setIndex >= G_SET_FIRST_SLEEPING )
		gsolver_set_wake( w, bodyA->setIndex );
	int islandIdA = bodyA->islandId;
	int islandIdB = bodyB->islandId;
	if ( islandIdA == islandIdB )
	{
		push_contact( w, islandIdA, c );
		return;
	}
	push_contact( w, link_islands( w, islandIdA, islandIdB ), c );
}

void gisland_unlink_contact( gWorld* w, gContact* c )
{
	gIsland* island = w->islands + c->islandId;
	if ( c->islandPrev != B2G_NULL )
		w->contacts[c->islandPrev].islandNext = c->islandNext;
	if ( c->islandNext != B2G_NULL )
		w->contacts[c->islandNext].islandPrev = c->islandPrev;
	if ( island->headContact == c->id )
		island->headContact = c->islandNext;
	if ( island->tailContact == c->id )
		island->tailContact = c->islandPrev;
	island->contactCount -= 1;
	island->constraintRemoveCount += 1;
	c->islandId = B2G_NULL;
	c->islandPrev = B2G_NULL;
	c->islandNext = B2G_NULL;
}

void gisland_link_joint( gWorld* w, gJoint* j )
{
	gBody* bodyA = w->bodies + j->edges[0].bodyId;
	gBody* bodyB = w->bodies + j->edges[1].bodyId;
	if ( bodyA->setIndex == G_SET_AWAKE && bodyB->setIndex >= G_SET_FIRST_SLEEPING )
		gsolver_set_wake( w, bodyB->setIndex );
	else if ( bodyB->setIndex == G_SET_AWAKE && bodyA->setIndex >= G_SET_FIRST_SLEEPING )
		gsolver_set_wake( w, bodyA->setIndex );
	int islandIdA = bodyA->islandId;
	int islandIdB = bodyB->islandId;
	if ( islandIdA == islandIdB )
	{
		push_joint( w, islandIdA, j );
		return;
	}
	push_joint( w, link_islands( w, islandIdA, islandIdB ), j );
}

void gisland_unlink_joint( gWorld* w, gJoint* j )
{
	if ( j->islandId == B2G_NULL )
		return;
	gIsland* island = w->islands + j->islandId;
	if ( j->islandPrev != B2G_NULL )
		w->joints[j->islandPrev].islandNext = j->islandNext;
	if ( j->islandNext != B2G_NULL )
		w->joints[j->islandNext].islandPrev = j->islandPrev;
	if ( island->headJoint == j->id )
		island->headJoint = j->islandNext;
	if ( island->tailJoint == j->id )
		island->tailJoint = j->islandPrev;
	island->jointCount -= 1;
	island->constraintRemoveCount += 1;
	j->islandId = B2G_NULL;
	j->islandPrev = B2G_NULL;
	j->islandNext = B2G_NULL;
}

/* Appends an island's lists to its root's (reference src/island.c:428-540). */
static void merge_into_root( gWorld* w, gIsland* island )
{
	int rootId = island->parentIsland;
	gIsland* root = w->islands + rootId;
	for ( int b = island->headBody; b != B2G_NULL; b = w->bodies[b].islandNext )
		w->bodies[b].islandId = rootId;
	for ( int c = island->headContact; c != B2G_NULL; c = w->contacts[c].islandNext )
		w->contacts[c].islandId = rootId;
	for ( int j = island->headJoint; j != B2G_NULL; j = w->joints[j].islandNext )
		w->joints[j].islandId = rootId;

	w->bodies[root->tailBody].islandNext = island->headBody;
	w->bodies[island->headBody].islandPrev = root->tailBody;
	root->tailBody = island->tailBody;
	root->bodyCount += island->bodyCount;

	if ( root->headContact == B2G_NULL )
	{
		root->headContact = island->headContact;
		root->tailContact = island->tailContact;
		root->contactCount = island->contactCount;
	}
	else if ( island->headContact != B2G_NULL )
	{
		w->contacts[root->tailContact].islandNext = island->headContact;
		w->contacts[island->headContact].islandPrev = root->tailContact;
		root->tailContact = island->tailContact;
		root->contactCount += island->contactCount;
	}

	if ( root->headJoint == B2G_NULL )
	{
		root->headJoint = island->headJoint;
		root->tailJoint = island->tailJoint;
		root->jointCount = island->jointCount;
	}
	else if ( island->headJoint != B2G_NULL )
	{
		w->joints[root->tailJoint].islandNext = island->headJoint;
		w->joints[island->headJoint].islandPrev = root->tailJoint;
		root->tailJoint = island->tailJoint;
		root->jointCount += island->jointCount;
	}
	root->constraintRemoveCount += island->constraintRemoveCount;
}

void gislands_merge_awake( gWorld* w )
{
	int count = w->awakeIslands.count;
	/* every child points at its root first, so that no child merges into an island that
	 * itself merges away */
	for ( int i = 0; i < count; ++i )
	{
		int islandId = w->awakeIslands.data[i];
		int rootId = island_root( w, islandId );
		if ( rootId != islandId )
			w->islands[islandId].parentIsland = rootId;
	}
	/* in reverse, because destroying an island swaps the last one into its place */
	for ( int i = count - 1; i >= 0; --i )
	{
		int islandId = w->awakeIslands.data[i];
		gIsland* island = w->islands + islandId;
		if ( island->parentIsland == B2G_NULL )
			continue;
		merge_into_root( w, island );
		destroy_island( w, islandId );
	}
}

/* Splits an awake island whose constraints were removed into its connected parts, by
 * depth-first search from each unvisited body in island order (reference
 * src/island.c:609-865). */
void gisland_split( gWorld* w, int baseId )
{
	gIsland* base = w->islands + baseId;
	int setIndex = base->setIndex;
	if ( setIndex != G_SET_AWAKE || base->constraintRemoveCount == 0 )
		return;
	int bodyCount = base->bodyCount;
	int* stack = (int*)b2g_alloc( sizeof( int ) * (size_t)( bodyCount > 0 ? bodyCount : 1 ) );
	int* bodyIds = (int*)b2g_alloc( sizeof( int ) * (size_t)( bodyCount > 0 ? bodyCount : 1 ) );
	if ( stack == NULL || bodyIds == NULL )
	{
		b2g_free( stack );
		b2g_free( bodyIds );
		return;
	}
	int n = 0;
	for ( int b = base->headBody; b != B2G_NULL; b = w->bodies[b].islandNext )
	{
		bodyIds[n++] = b;
		w->bodies[b].isMarked = false;
	}
	for ( int c = base->headContact; c != B2G_NULL; c = w->contacts[c].islandNext )
		w->contacts[c].isMarked = false;
	for ( int j = base->headJoint; j != B2G_NULL; j = w->joints[j].islandNext )
		w->joints[j].isMarked = false;
	destroy_island( w, baseId );

	for ( int i = 0; i < bodyCount; ++i )
	{
		gBody* seed = w->bodies + bodyIds[i];
		if ( seed->isMarked )
			continue;
		int top = 0;
		stack[top++] = seed->id;
		seed->isMarked = true;
		gIsland* island = create_island( w, setIndex );
		if ( island == NULL )
			break;
		int islandId = island->islandId;
		while ( top > 0 )
		{
			int bodyId = stack[--top];
			gBody* body = w->bodies + bodyId;
			body->islandId = islandId;
			if ( island->tailBody != B2G_NULL )
				w->bodies[island->tailBody].islandNext = bodyId;
			body->islandPrev = island->tailBody;
			body->islandNext = B2G_NULL;
			island->tailBody = bodyId;
			if ( island->headBody == B2G_NULL )
				island->headBody = bodyId;
			island->bodyCount += 1;

			for ( int key = body->headContactKey; key != B2G_NULL; )
			{
				int contactId = key >> 1;
				int edge = key & 1;
				gContact* c = w->contacts + contactId;
				key = c->edges[edge].nextKey;
				if ( c->isMarked || ( c->flags & G_SENSOR ) || ( c->flags & G_TOUCHING ) == 0 )
					continue;
				c->isMarked = true;
				gBody* other = w->bodies + c->edges[edge ^ 1].bodyId;
				if ( other->isMarked == false && other->setIndex != G_SET_STATIC )
				{
					stack[top++] = other->id;
					other->isMarked = true;
				}
				c->islandId = islandId;
				if ( island->tailContact != B2G_NULL )
					w->contacts[island->tailContact].islandNext = contactId;
				c->islandPrev = island->tailContact;
				c->islandNext = B2G_NULL;
				island->tailContact = contactId;
				if ( island->headContact == B2G_NULL )
					island->headContact = contactId;
				island->contactCount += 1;
			}

			for ( int key = body->headJointKey; key != B2G_NULL; )
			{
				int jointId = key >> 1;
				int edge = key & 1;
				gJoint* j = w->joints + jointId;
				key = j->edges[edge].nextKey;
				if ( j->isMarked )
					continue;
				j->isMarked = true;
				gBody* other = w->bodies + j->edges[edge ^ 1].bodyId;
				if ( other->setIndex == G_SET_DISABLED )
					continue;
				if ( other->isMarked == false && other->setIndex == G_SET_AWAKE )
				{
					stack[top++] = other->id;
					other->isMarked = true;
				}
				j->islandId = islandId;
				if ( island->tailJoint != B2G_NULL )
					w->joints[island->tailJoint].islandNext = jointId;
				j->islandPrev = island->tailJoint;
				j->islandNext = B2G_NULL;
				island->tailJoint = jointId;
				if ( island->headJoint == B2G_NULL )
					island->headJoint = jointId;
				island->jointCount += 1;
			}
		}
	}
	b2g_free( bodyIds );
	b2g_free( stack );
}

/* ------------------------------------------------------------ solver sets */
int gsolver_set_create( gWorld* w )
{
	int setId = gid_alloc( &w->setIds );
	if ( grow_sets( w, setId + 1 ) == false )
	{
		gid_unalloc( &w->setIds, setId );
		return B2G_NULL;
	}
	gSolverSet* set = w->sets + setId;
	set->setIndex = setId;
	set->bodies.count = 0;
	set->contacts.count = 0;
	set->joints.count = 0;
	set->islands.count = 0;
	return setId;
}

static void destroy_set( gWorld* w, int setIndex )
{
	gSolverSet* set = w->sets + setIndex;
	set->bodies.count = 0;
	set->contacts.count = 0;
	set->joints.count = 0;
	set->islands.count = 0;
	set->setIndex = B2G_NULL;
	gid_free( &w->setIds, setIndex );
}

static void joint_to_graph( gWorld* w, gJoint* j )
{
	bool staticA = w->bodies[j->bodyIdA].setIndex == G_SET_STATIC;
	bool staticB = w->bodies[j->bodyIdB].setIndex == G_SET_STATIC;
	int color = gassign_joint_color( w, j->bodyIdA, j->bodyIdB, staticA, staticB );
	j->colorIndex = color;
	j->localIndex = w->colors[color].joints.count;
	gia_push( &w->colors[color].joints, j->id );
	w->solveDirty = true;
}

/* Wakes a sleeping set: bodies join the awake list with the identity state, their
 * contacts of the disabled set rejoin the awake set, the set's touching contacts and
 * joints rejoin the graph and its islands the awake islands (reference
 * src/solver_set.c:35-160). */
void gsolver_set_wake( gWorld* w, int setIndex )
{
	gSolverSet* set = w->sets + setIndex;
	for ( int i = 0; i < set->bodies.count; ++i )
	{
		gBody* body = w->bodies + set->bodies.data[i];
		body->setIndex = G_SET_AWAKE;
		body->setLocal = B2G_NULL;
		body->awakeIndex = w->awake.count;
		gia_push( &w->awake, body->id );
		w->awakeDirty = true;
		gbody_stage_op( w, body->id, B2G_BODY_WAKE );
		for ( int key = body->headContactKey; key != B2G_NULL; )
		{
			int edge = key & 1;
			gContact* c = w->contacts + ( key >> 1 );
			key = c->edges[edge].nextKey;
			if ( c->setIndex != G_SET_DISABLED )
				continue;
			int localIndex = c->localIndex;
			c->setIndex = G_SET_AWAKE;
			c->localIndex = w->nonTouching.count;
			gia_push( &w->nonTouching, c->id );
			int moved = gia_remove_swap( &w->disabledContacts, localIndex );
			if ( moved != B2G_NULL )
				w->contacts[w->disabledContacts.data[localIndex]].localIndex = localIndex;
			gcontact_stage_set( w, c->id, false );
		}
	}
	for ( int i = 0; i < set->contacts.count; ++i )
	{
		gContact* c = w->contacts + set->contacts.data[i];
		gcontact_add_to_graph( w, c );
		c->setIndex = G_SET_AWAKE;
		gcontact_stage_set( w, c->id, false );
	}
	for ( int i = 0; i < set->joints.count; ++i )
	{
		gJoint* j = w->joints + set->joints.data[i];
		joint_to_graph( w, j );
		j->setIndex = G_SET_AWAKE;
	}
	for ( int i = 0; i < set->islands.count; ++i )
	{
		gIsland* island = w->islands + set->islands.data[i];
		island->setIndex = G_SET_AWAKE;
		island->localIndex = w->awakeIslands.count;
		gia_push( &w->awakeIslands, island->islandId );
	}
	destroy_set( w, setIndex );
}

/* Moves an island into a new sleeping set, unless constraints were removed from it since
 * its last split (reference src/solver_set.c:162-451). */
void gisland_try_sleep( gWorld* w, int islandId )
{
	gIsland* island = w->islands + islandId;
	if ( island->constraintRemoveCount > 0 )
		return;
	int sleepSetId = gsolver_set_create( w );
	if ( sleepSetId == B2G_NULL )
		return;
	gSolverSet* sleepSet = w->sets + sleepSetId;

	for ( int bodyId = island->headBody; bodyId != B2G_NULL; )
	{
		gBody* body = w->bodies + bodyId;
		int awakeIndex = body->awakeIndex;
		int sleepIndex = sleepSet->bodies.count;
		gia_push( &sleepSet->bodies, bodyId );
		int moved = gia_remove_swap( &w->awake, awakeIndex );
		if ( moved != B2G_NULL )
			w->bodies[w->awake.data[awakeIndex]].awakeIndex = awakeIndex;
		w->awakeDirty = true;
		body->setIndex = sleepSetId;
		body->awakeIndex = B2G_NULL;
		body->setLocal = sleepIndex;
		gbody_stage_op( w, bodyId, B2G_BODY_SLEEP );

		/* non-touching contacts whose other body is not awake either leave the awake set */
		for ( int key = body->headContactKey; key != B2G_NULL; )
		{
			int edge = key & 1;
			gContact* c = w->contacts + ( key >> 1 );
			key = c->edges[edge].nextKey;
			if ( c->setIndex == G_SET_DISABLED || c->colorIndex != B2G_NULL )
				continue;
			if ( w->bodies[c->edges[edge ^ 1].bodyId].setIndex == G_SET_AWAKE )
				continue;
			int localIndex = c->localIndex;
			c->setIndex = G_SET_DISABLED;
			c->localIndex = w->disabledContacts.count;
			gia_push( &w->disabledContacts, c->id );
			int movedContact = gia_remove_swap( &w->nonTouching, localIndex );
			if ( movedContact != B2G_NULL )
				w->contacts[w->nonTouching.data[localIndex]].localIndex = localIndex;
			gcontact_stage_set( w, c->id, true );
		}
		bodyId = body->islandNext;
	}

	/* touching contacts leave the graph */
	for ( int contactId = island->headContact; contactId != B2G_NULL; )
	{
		gContact* c = w->contacts + contactId;
		int sleepIndex = sleepSet->contacts.count;
		gia_push( &sleepSet->contacts, contactId );
		gcontact_remove_from_graph( w, c->edges[0].bodyId, c->edges[1].bodyId, c->colorIndex, c->localIndex );
		c->setIndex = sleepSetId;
		c->colorIndex = B2G_NULL;
		c->localIndex = sleepIndex;
		gcontact_stage_set( w, contactId, true );
		contactId = c->islandNext;
	}

	/* joints leave the graph */
	for ( int jointId = island->headJoint; jointId != B2G_NULL; )
	{
		gJoint* j = w->joints + jointId;
		gColor* color = w->colors + j->colorIndex;
		if ( j->colorIndex != B2G_OVERFLOW )
		{
			gbits_clear( &color->bodySet, j->edges[0].bodyId );
			gbits_clear( &color->bodySet, j->edges[1].bodyId );
		}
		int sleepIndex = sleepSet->joints.count;
		gia_push( &sleepSet->joints, jointId );
		int moved = gia_remove_swap( &color->joints, j->localIndex );
		if ( moved != B2G_NULL )
			w->joints[color->joints.data[j->localIndex]].localIndex = j->localIndex;
		w->solveDirty = true;
		j->setIndex = sleepSetId;
		j->colorIndex = B2G_NULL;
		j->localIndex = sleepIndex;
		jointId = j->islandNext;
	}

	int islandIndex = island->localIndex;
	gia_push( &sleepSet->islands, islandId );
	int moved = gia_remove_swap( &w->awakeIslands, islandIndex );
	if ( moved != B2G_NULL )
		w->islands[w->awakeIslands.data[islandIndex]].localIndex = islandIndex;
	island->setIndex = sleepSetId;
	island->localIndex = 0;
}

/* Merges the smaller of two sleeping sets into the larger (reference
 * src/solver_set.c:456-554). */
void gsolver_set_merge( gWorld* w, int setId1, int setId2 )
{
	if ( w->sets[setId1].bodies.count < w->sets[setId2].bodies.count )
	{
		int t = setId1;
		setId1 = setId2;
		setId2 = t;
	}
	gSolverSet* set1 = w->sets + setId1;
	gSolverSet* set2 = w->sets + setId2;
	for ( int i = 0; i < set2->bodies.count; ++i )
	{
		gBody* body = w->bodies + set2->bodies.data[i];
		body->setIndex = setId1;
		body->setLocal = set1->bodies.count;
		gia_push( &set1->bodies, body->id );
	}
	for ( int i = 0; i < set2->contacts.count; ++i )
	{
		gContact* c = w->contacts + set2->contacts.data[i];
		c->setIndex = setId1;
		c->localIndex = set1->contacts.count;
		gia_push( &set1->contacts, c->id );
	}
	for ( int i = 0; i < set2->joints.count; ++i )
	{
		gJoint* j = w->joints + set2->joints.data[i];
		j->setIndex = setId1;
		j->localIndex = set1->joints.count;
		gia_push( &set1->joints, j->id );
	}
	for ( int i = 0; i < set2->islands.count; ++i )
	{
		gIsland* island = w->islands + set2->islands.data[i];
		island->setIndex = setId1;
		island->localIndex = set1->islands.count;
		gia_push( &set1->islands, island->islandId );
	}
	destroy_set( w, setId2 );
}

bool gbody_wake( gWorld* w, gBody* b )
{
	if ( b->setIndex >= G_SET_FIRST_SLEEPING )
	{
		gsolver_set_wake( w, b->setIndex );
		return true;
	}
	return false;
}

/* ------------------------------------------------------------ end of step */
void gislands_sleep_step( gWorld* w )
{
	if ( w->enableSleep == false )
		return;
	int islandCount = w->awakeIslands.count;
	if ( islandCount > w->islandSleepyCap )
	{
		int nc = w->islandSleepyCap < 64 ? 64 : w->islandSleepyCap;
		while ( nc < islandCount )
			nc *= 2;
		int* p = (int*)b2g_realloc( w->islandSleepy, sizeof( int ) * (size_t)nc );
		if ( p == NULL )
			return;
		w->islandSleepy = p;
		w->islandSleepyCap = nc;
	}
	if ( islandCount > 0 )
		memset( w->islandSleepy, 0, sizeof( int ) * (size_t)islandCount );

	/* every body below the sleep time keeps its island awake; among the rest, the first
	 * body in awake order with the longest sleep time picks the island to split next */
	int n = w->io.counters[3];
	n = n < w->dev.sleepyCap ? n : w->dev.sleepyCap;
	w->dev.d2hBytes += 8 * (long long)n;
	int split = B2G_NULL, splitIndex = 0;
	float splitTime = 0.0f;
	for ( int r = 0; r < n; ++r )
	{
		int awakeIndex = w->io.sleepy[2 * r];
		float t;
		memcpy( &t, w->io.sleepy + 2 * r + 1, sizeof( float ) );
		if ( awakeIndex < 0 || awakeIndex >= w->awake.count )
			continue;
		gBody* b = w->bodies + w->awake.data[awakeIndex];
		gIsland* island = w->islands + b->islandId;
		w->islandSleepy[island->localIndex] += 1;
		if ( island->constraintRemoveCount > 0 && ( t > splitTime || ( t == splitTime && awakeIndex < splitIndex ) ) )
		{
			split = b->islandId;
			splitTime = t;
			splitIndex = awakeIndex;
		}
	}
	w->splitIslandId = split;

	/* in reverse, because a sleeping island's place is taken by the last one */
	for ( int k = islandCount - 1; k >= 0; --k )
	{
		int islandId = w->awakeIslands.data[k];
		if ( w->islandSleepy[k] == w->islands[islandId].bodyCount )
			gisland_try_sleep( w, islandId );
	}
}
