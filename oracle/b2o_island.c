/*
 * b2o_island.c -- persistent islands, solver sets and sleep for the plain-C oracle
 * (TEST INFRASTRUCTURE).
 *
 * Restates the reference: src/island.c:16-865 (island creation and destruction, contact
 * and joint linking with union-find, merging awake islands, splitting an island by
 * depth-first search), src/solver_set.c:16-554 (waking a sleeping set, putting an island
 * to sleep, merging two sleeping sets) and src/body.c:84-159, :325-333 (a body's own
 * island, leaving an island, waking a body).  The order in which bodies, contacts and
 * joints move between sets fixes the awake order, the colours and the contact ids of
 * later steps, so every loop keeps the reference's order.
 *
 * Set membership: the awake set's bodies are w->awake (body->awakeIndex), its non-touching
 * contacts w->nonTouching and its touching contacts and joints the graph colours; the
 * disabled set holds non-touching contacts whose bodies both sleep; a sleeping set keeps
 * its members in w->sets[id] (body->setLocal, contact and joint localIndex).
 */
#include "b2o.h"

#include <stdlib.h>
#include <string.h>

#define GROWN( ptr, cap, need, T )                                                                                               \
	do                                                                                                                           \
	{                                                                                                                            \
		if ( ( need ) > ( cap ) )                                                                                                \
		{                                                                                                                        \
			int nc = ( cap ) < 16 ? 16 : ( cap );                                                                                \
			while ( nc < ( need ) )                                                                                              \
				nc *= 2;                                                                                                         \
			ptr = (T*)realloc( ptr, sizeof( T ) * (size_t)nc );                                                                  \
			memset( ptr + ( cap ), 0, sizeof( T ) * (size_t)( nc - ( cap ) ) );                                                 \
			cap = nc;                                                                                                            \
		}                                                                                                                        \
	} while ( 0 )

void o_islands_init( oWorld* w )
{
	/* set ids 0, 1 and 2 are the static, disabled and awake sets (reference world.c:140-160) */
	for ( int i = 0; i < O_SET_FIRST_SLEEPING; ++i )
		oid_alloc( &w->setIds );
	GROWN( w->sets, w->setCap, O_SET_FIRST_SLEEPING, oSolverSet );
	for ( int i = 0; i < O_SET_FIRST_SLEEPING; ++i )
		w->sets[i].setIndex = i;
	w->splitIslandId = O_NULL;
}

void o_islands_free( oWorld* w )
{
	for ( int i = 0; i < w->setCap; ++i )
	{
		oia_free( &w->sets[i].bodies );
		oia_free( &w->sets[i].contacts );
		oia_free( &w->sets[i].joints );
		oia_free( &w->sets[i].islands );
	}
	free( w->sets );
	free( w->islands );
	oia_free( &w->islandIds.freeIds );
	oia_free( &w->setIds.freeIds );
	oia_free( &w->awakeIslands );
	oia_free( &w->disabledContacts );
}

oIntArray* o_set_bodies( oWorld* w, int setIndex )
{
	if ( setIndex == O_SET_AWAKE )
		return &w->awake;
	if ( setIndex == O_SET_STATIC )
		return &w->staticBodies;
	return &w->sets[setIndex].bodies;
}

oIntArray* o_set_contacts( oWorld* w, int setIndex )
{
	if ( setIndex == O_SET_AWAKE )
		return &w->nonTouching;
	if ( setIndex == O_SET_DISABLED )
		return &w->disabledContacts;
	return &w->sets[setIndex].contacts;
}

oIntArray* o_set_joints( oWorld* w, int setIndex ) { return &w->sets[setIndex].joints; }

static oIntArray* set_islands( oWorld* w, int setIndex )
{
	return setIndex == O_SET_AWAKE ? &w->awakeIslands : &w->sets[setIndex].islands;
}

/* body position within its set */
static int body_local( const oBody* b ) { return b->setIndex == O_SET_AWAKE ? b->awakeIndex : b->setLocal; }
static void set_body_local( oBody* b, int index )
{
	if ( b->setIndex == O_SET_AWAKE )
	{
		b->awakeIndex = index;
		b->setLocal = O_NULL;
	}
	else
	{
		b->awakeIndex = O_NULL;
		b->setLocal = index;
	}
}

/* Swap-removes a body from its set's list, fixing the moved body's index. */
void o_remove_body_from_set( oWorld* w, oBody* b )
{
	oIntArray* list = o_set_bodies( w, b->setIndex );
	int local = body_local( b );
	int moved = oia_remove_swap( list, local );
	if ( moved != O_NULL )
		set_body_local( w->bodies + list->data[local], local );
}

/* ------------------------------------------------------------ islands */
/* reference src/island.c:16-55 */
static oIsland* create_island( oWorld* w, int setIndex )
{
	int islandId = oid_alloc( &w->islandIds );
	GROWN( w->islands, w->islandCap, islandId + 1, oIsland );
	oIntArray* list = set_islands( w, setIndex );
	oIsland* island = w->islands + islandId;
	island->setIndex = setIndex;
	island->localIndex = list->count;
	island->islandId = islandId;
	island->headBody = O_NULL;
	island->tailBody = O_NULL;
	island->bodyCount = 0;
	island->headContact = O_NULL;
	island->tailContact = O_NULL;
	island->contactCount = 0;
	island->headJoint = O_NULL;
	island->tailJoint = O_NULL;
	island->jointCount = 0;
	island->parentIsland = O_NULL;
	island->constraintRemoveCount = 0;
	oia_push( list, islandId );
	return island;
}

/* reference src/island.c:57-80 */
static void destroy_island( oWorld* w, int islandId )
{
	oIsland* island = w->islands + islandId;
	oIntArray* list = set_islands( w, island->setIndex );
	int moved = oia_remove_swap( list, island->localIndex );
	if ( moved != O_NULL )
		w->islands[list->data[island->localIndex]].localIndex = island->localIndex;
	island->islandId = O_NULL;
	island->setIndex = O_NULL;
	island->localIndex = O_NULL;
	oid_free( &w->islandIds, islandId );
}

/* reference src/body.c:84-97 */
void o_create_island_for_body( oWorld* w, int setIndex, oBody* b )
{
	oIsland* island = create_island( w, setIndex );
	b->islandId = island->islandId;
	island->headBody = b->id;
	island->tailBody = b->id;
	island->bodyCount = 1;
}

/* reference src/body.c:99-159 */
void o_remove_body_from_island( oWorld* w, oBody* b )
{
	if ( b->islandId == O_NULL )
		return;
	int islandId = b->islandId;
	oIsland* island = w->islands + islandId;
	if ( b->islandPrev != O_NULL )
		w->bodies[b->islandPrev].islandNext = b->islandNext;
	if ( b->islandNext != O_NULL )
		w->bodies[b->islandNext].islandPrev = b->islandPrev;
	island->bodyCount -= 1;
	if ( island->headBody == b->id )
	{
		island->headBody = b->islandNext;
		if ( island->headBody == O_NULL )
			destroy_island( w, island->islandId );
	}
	else if ( island->tailBody == b->id )
		island->tailBody = b->islandPrev;
	b->islandId = O_NULL;
	b->islandPrev = O_NULL;
	b->islandNext = O_NULL;
}

/* reference src/island.c:88-118 */
static void add_contact_to_island( oWorld* w, int islandId, oContact* c )
{
	oIsland* island = w->islands + islandId;
	if ( island->headContact != O_NULL )
	{
		c->islandNext = island->headContact;
		w->contacts[island->headContact].islandPrev = c->id;
	}
	island->headContact = c->id;
	if ( island->tailContact == O_NULL )
		island->tailContact = island->headContact;
	island->contactCount += 1;
	c->islandId = islandId;
}

/* reference src/island.c:120-221 */
void o_link_contact( oWorld* w, oContact* c )
{
	oBody* bodyA = w->bodies + c->edges[0].bodyId;
	oBody* bodyB = w->bodies + c->edges[1].bodyId;
	if ( bodyA->setIndex == O_SET_AWAKE && bodyB->setIndex >= O_SET_FIRST_SLEEPING )
		o_wake_solver_set( w, bodyB->setIndex );
	if ( bodyB->setIndex == O_SET_AWAKE && bodyA->setIndex >= O_SET_FIRST_SLEEPING )
		o_wake_solver_set( w, bodyA->setIndex );

	int islandIdA = bodyA->islandId;
	int islandIdB = bodyB->islandId;
	if ( islandIdA == islandIdB )
	{
		add_contact_to_island( w, islandIdA, c );
		return;
	}

	oIsland* islandA = NULL;
	if ( islandIdA != O_NULL )
	{
		islandA = w->islands + islandIdA;
		int parentId = islandA->parentIsland;
		while ( parentId != O_NULL )
		{
			oIsland* parent = w->islands + parentId;
			if ( parent->parentIsland != O_NULL )
				islandA->parentIsland = parent->parentIsland;
			islandA = parent;
			islandIdA = parentId;
			parentId = islandA->parentIsland;
		}
	}

	oIsland* islandB = NULL;
	if ( islandIdB != O_NULL )
	{
		islandB = w->islands + islandIdB;
		int parentId = islandB->parentIsland;
		while ( islandB->parentIsland != O_NULL )
		{
			oIsland* parent = w->islands + parentId;
			if ( parent->parentIsland != O_NULL )
				islandB->parentIsland = parent->parentIsland;
			islandB = parent;
			islandIdB = parentId;
			parentId = islandB->parentIsland;
		}
	}

	if ( islandA != islandB && islandA != NULL && islandB != NULL )
		islandB->parentIsland = islandIdA;

	if ( islandA != NULL )
		add_contact_to_island( w, islandIdA, c );
	else
		add_contact_to_island( w, islandIdB, c );
}

/* reference src/island.c:223-268 */
void o_unlink_contact( oWorld* w, oContact* c )
{
	int islandId = c->islandId;
	oIsland* island = w->islands + islandId;
	if ( c->islandPrev != O_NULL )
		w->contacts[c->islandPrev].islandNext = c->islandNext;
	if ( c->islandNext != O_NULL )
		w->contacts[c->islandNext].islandPrev = c->islandPrev;
	if ( island->headContact == c->id )
		island->headContact = c->islandNext;
	if ( island->tailContact == c->id )
		island->tailContact = c->islandPrev;
	island->contactCount -= 1;
	island->constraintRemoveCount += 1;
	c->islandId = O_NULL;
	c->islandPrev = O_NULL;
	c->islandNext = O_NULL;
}

/* reference src/island.c:270-296 */
static void add_joint_to_island( oWorld* w, int islandId, oJoint* j )
{
	oIsland* island = w->islands + islandId;
	if ( island->headJoint != O_NULL )
	{
		j->islandNext = island->headJoint;
		w->joints[island->headJoint].islandPrev = j->id;
	}
	island->headJoint = j->id;
	if ( island->tailJoint == O_NULL )
		island->tailJoint = island->headJoint;
	island->jointCount += 1;
	j->islandId = islandId;
}

/* reference src/island.c:298-380 */
void o_link_joint( oWorld* w, oJoint* j )
{
	oBody* bodyA = w->bodies + j->edges[0].bodyId;
	oBody* bodyB = w->bodies + j->edges[1].bodyId;
	if ( bodyA->setIndex == O_SET_AWAKE && bodyB->setIndex >= O_SET_FIRST_SLEEPING )
		o_wake_solver_set( w, bodyB->setIndex );
	else if ( bodyB->setIndex == O_SET_AWAKE && bodyA->setIndex >= O_SET_FIRST_SLEEPING )
		o_wake_solver_set( w, bodyA->setIndex );

	int islandIdA = bodyA->islandId;
	int islandIdB = bodyB->islandId;
	if ( islandIdA == islandIdB )
	{
		add_joint_to_island( w, islandIdA, j );
		return;
	}

	oIsland* islandA = NULL;
	if ( islandIdA != O_NULL )
	{
		islandA = w->islands + islandIdA;
		while ( islandA->parentIsland != O_NULL )
		{
			oIsland* parent = w->islands + islandA->parentIsland;
			if ( parent->parentIsland != O_NULL )
				islandA->parentIsland = parent->parentIsland;
			islandIdA = islandA->parentIsland;
			islandA = parent;
		}
	}

	oIsland* islandB = NULL;
	if ( islandIdB != O_NULL )
	{
		islandB = w->islands + islandIdB;
		while ( islandB->parentIsland != O_NULL )
		{
			oIsland* parent = w->islands + islandB->parentIsland;
			if ( parent->parentIsland != O_NULL )
				islandB->parentIsland = parent->parentIsland;
			islandIdB = islandB->parentIsland;
			islandB = parent;
		}
	}

	if ( islandA != islandB && islandA != NULL && islandB != NULL )
		islandB->parentIsland = islandIdA;

	if ( islandA != NULL )
		add_joint_to_island( w, islandIdA, j );
	else
		add_joint_to_island( w, islandIdB, j );
}

/* reference src/island.c:382-426 */
void o_unlink_joint( oWorld* w, oJoint* j )
{
	if ( j->islandId == O_NULL )
		return;
	int islandId = j->islandId;
	oIsland* island = w->islands + islandId;
	if ( j->islandPrev != O_NULL )
		w->joints[j->islandPrev].islandNext = j->islandNext;
	if ( j->islandNext != O_NULL )
		w->joints[j->islandNext].islandPrev = j->islandPrev;
	if ( island->headJoint == j->id )
		island->headJoint = j->islandNext;
	if ( island->tailJoint == j->id )
		island->tailJoint = j->islandPrev;
	island->jointCount -= 1;
	island->constraintRemoveCount += 1;
	j->islandId = O_NULL;
	j->islandPrev = O_NULL;
	j->islandNext = O_NULL;
}

/* reference src/island.c:428-540 */
static void merge_island( oWorld* w, oIsland* island )
{
	int rootId = island->parentIsland;
	oIsland* root = w->islands + rootId;

	for ( int b = island->headBody; b != O_NULL; b = w->bodies[b].islandNext )
		w->bodies[b].islandId = rootId;
	for ( int c = island->headContact; c != O_NULL; c = w->contacts[c].islandNext )
		w->contacts[c].islandId = rootId;
	for ( int j = island->headJoint; j != O_NULL; j = w->joints[j].islandNext )
		w->joints[j].islandId = rootId;

	w->bodies[root->tailBody].islandNext = island->headBody;
	w->bodies[island->headBody].islandPrev = root->tailBody;
	root->tailBody = island->tailBody;
	root->bodyCount += island->bodyCount;

	if ( root->headContact == O_NULL )
	{
		root->headContact = island->headContact;
		root->tailContact = island->tailContact;
		root->contactCount = island->contactCount;
	}
	else if ( island->headContact != O_NULL )
	{
		w->contacts[root->tailContact].islandNext = island->headContact;
		w->contacts[island->headContact].islandPrev = root->tailContact;
		root->tailContact = island->tailContact;
		root->contactCount += island->contactCount;
	}

	if ( root->headJoint == O_NULL )
	{
		root->headJoint = island->headJoint;
		root->tailJoint = island->tailJoint;
		root->jointCount = island->jointCount;
	}
	else if ( island->headJoint != O_NULL )
	{
		w->joints[root->tailJoint].islandNext = island->headJoint;
		w->joints[island->headJoint].islandPrev = root->tailJoint;
		root->tailJoint = island->tailJoint;
		root->jointCount += island->jointCount;
	}

	root->constraintRemoveCount += island->constraintRemoveCount;
}

/* reference src/island.c:542-607 */
void o_merge_awake_islands( oWorld* w )
{
	int count = w->awakeIslands.count;
	for ( int i = 0; i < count; ++i )
	{
		int islandId = w->awakeIslands.data[i];
		oIsland* island = w->islands + islandId;
		int rootId = islandId;
		oIsland* root = island;
		while ( root->parentIsland != O_NULL )
		{
			oIsland* parent = w->islands + root->parentIsland;
			if ( parent->parentIsland != O_NULL )
				root->parentIsland = parent->parentIsland;
			rootId = root->parentIsland;
			root = parent;
		}
		if ( root != island )
			island->parentIsland = rootId;
	}
	for ( int i = count - 1; i >= 0; --i )
	{
		int islandId = w->awakeIslands.data[i];
		oIsland* island = w->islands + islandId;
		if ( island->parentIsland == O_NULL )
			continue;
		merge_island( w, island );
		destroy_island( w, islandId );
	}
}

/* reference src/island.c:609-865 */
void o_split_island( oWorld* w, int baseId )
{
	oIsland* base = w->islands + baseId;
	int setIndex = base->setIndex;
	if ( setIndex != O_SET_AWAKE )
		return;
	if ( base->constraintRemoveCount == 0 )
		return;

	int bodyCount = base->bodyCount;
	int* stack = (int*)malloc( sizeof( int ) * (size_t)( bodyCount > 0 ? bodyCount : 1 ) );
	int* bodyIds = (int*)malloc( sizeof( int ) * (size_t)( bodyCount > 0 ? bodyCount : 1 ) );
	int index = 0;
	for ( int b = base->headBody; b != O_NULL; b = w->bodies[b].islandNext )
	{
		bodyIds[index++] = b;
		w->bodies[b].isMarked = false;
	}
	for ( int c = base->headContact; c != O_NULL; c = w->contacts[c].islandNext )
		w->contacts[c].isMarked = false;
	for ( int j = base->headJoint; j != O_NULL; j = w->joints[j].islandNext )
		w->joints[j].isMarked = false;

	destroy_island( w, baseId );

	for ( int i = 0; i < bodyCount; ++i )
	{
		int seedIndex = bodyIds[i];
		oBody* seed = w->bodies + seedIndex;
		if ( seed->isMarked )
			continue;
		int stackCount = 0;
		stack[stackCount++] = seedIndex;
		seed->isMarked = true;

		oIsland* island = create_island( w, setIndex );
		int islandId = island->islandId;

		while ( stackCount > 0 )
		{
			int bodyId = stack[--stackCount];
			oBody* body = w->bodies + bodyId;
			body->islandId = islandId;
			if ( island->tailBody != O_NULL )
				w->bodies[island->tailBody].islandNext = bodyId;
			body->islandPrev = island->tailBody;
			body->islandNext = O_NULL;
			island->tailBody = bodyId;
			if ( island->headBody == O_NULL )
				island->headBody = bodyId;
			island->bodyCount += 1;

			int contactKey = body->headContactKey;
			while ( contactKey != O_NULL )
			{
				int contactId = contactKey >> 1;
				int edgeIndex = contactKey & 1;
				oContact* c = w->contacts + contactId;
				contactKey = c->edges[edgeIndex].nextKey;
				if ( c->isMarked )
					continue;
				if ( c->flags & OC_SENSOR )
					continue;
				if ( ( c->flags & OC_TOUCHING ) == 0 )
					continue;
				c->isMarked = true;
				int otherBodyId = c->edges[edgeIndex ^ 1].bodyId;
				oBody* other = w->bodies + otherBodyId;
				if ( other->isMarked == false && other->setIndex != O_SET_STATIC )
				{
					stack[stackCount++] = otherBodyId;
					other->isMarked = true;
				}
				c->islandId = islandId;
				if ( island->tailContact != O_NULL )
					w->contacts[island->tailContact].islandNext = contactId;
				c->islandPrev = island->tailContact;
				c->islandNext = O_NULL;
				island->tailContact = contactId;
				if ( island->headContact == O_NULL )
					island->headContact = contactId;
				island->contactCount += 1;
			}

			int jointKey = body->headJointKey;
			while ( jointKey != O_NULL )
			{
				int jointId = jointKey >> 1;
				int edgeIndex = jointKey & 1;
				oJoint* j = w->joints + jointId;
				jointKey = j->edges[edgeIndex].nextKey;
				if ( j->isMarked )
					continue;
				j->isMarked = true;
				int otherBodyId = j->edges[edgeIndex ^ 1].bodyId;
				oBody* other = w->bodies + otherBodyId;
				if ( other->setIndex == O_SET_DISABLED )
					continue;
				if ( other->isMarked == false && other->setIndex == O_SET_AWAKE )
				{
					stack[stackCount++] = otherBodyId;
					other->isMarked = true;
				}
				j->islandId = islandId;
				if ( island->tailJoint != O_NULL )
					w->joints[island->tailJoint].islandNext = jointId;
				j->islandPrev = island->tailJoint;
				j->islandNext = O_NULL;
				island->tailJoint = jointId;
				if ( island->headJoint == O_NULL )
					island->headJoint = jointId;
				island->jointCount += 1;
			}
		}
	}
	free( bodyIds );
	free( stack );
}

/* ------------------------------------------------------------ solver sets */
int o_create_sleeping_set( oWorld* w )
{
	int setId = oid_alloc( &w->setIds );
	GROWN( w->sets, w->setCap, setId + 1, oSolverSet );
	oSolverSet* set = w->sets + setId;
	set->setIndex = setId;
	set->bodies.count = 0;
	set->contacts.count = 0;
	set->joints.count = 0;
	set->islands.count = 0;
	return setId;
}

/* reference src/solver_set.c:16-27 */
static void destroy_solver_set( oWorld* w, int setIndex )
{
	oSolverSet* set = w->sets + setIndex;
	set->bodies.count = 0;
	set->contacts.count = 0;
	set->joints.count = 0;
	set->islands.count = 0;
	set->setIndex = O_NULL;
	oid_free( &w->setIds, setIndex );
}

/* reference src/solver_set.c:35-160 */
void o_wake_solver_set( oWorld* w, int setIndex )
{
	oSolverSet* set = w->sets + setIndex;
	for ( int i = 0; i < set->bodies.count; ++i )
	{
		oBody* body = w->bodies + set->bodies.data[i];
		body->setIndex = O_SET_AWAKE;
		body->awakeIndex = w->awake.count;
		body->setLocal = O_NULL;
		oia_push( &w->awake, body->id );
		body->sleepTime = 0;
		/* a woken body starts from the identity state: no velocity, no deltas */
		body->v = ov( 0, 0 );
		body->w = 0;
		body->dp = ov( 0, 0 );
		body->dq = orot( 1, 0 );

		/* non-touching contacts of the disabled set join the awake set */
		int contactKey = body->headContactKey;
		while ( contactKey != O_NULL )
		{
			int edgeIndex = contactKey & 1;
			oContact* c = w->contacts + ( contactKey >> 1 );
			contactKey = c->edges[edgeIndex].nextKey;
			if ( c->setIndex != O_SET_DISABLED )
				continue;
			int localIndex = c->localIndex;
			c->setIndex = O_SET_AWAKE;
			c->localIndex = w->nonTouching.count;
			oia_push( &w->nonTouching, c->id );
			int moved = oia_remove_swap( &w->disabledContacts, localIndex );
			if ( moved != O_NULL )
				w->contacts[w->disabledContacts.data[localIndex]].localIndex = localIndex;
		}
	}
	for ( int i = 0; i < set->contacts.count; ++i )
	{
		oContact* c = w->contacts + set->contacts.data[i];
		o_add_contact_to_graph( w, c );
		c->setIndex = O_SET_AWAKE;
	}
	for ( int i = 0; i < set->joints.count; ++i )
	{
		oJoint* j = w->joints + set->joints.data[i];
		bool staticA = w->bodies[j->bodyIdA].setIndex == O_SET_STATIC;
		bool staticB = w->bodies[j->bodyIdB].setIndex == O_SET_STATIC;
		int color = o_assign_joint_color( w, j->bodyIdA, j->bodyIdB, staticA, staticB );
		j->colorIndex = color;
		j->localIndex = w->colors[color].joints.count;
		oia_push( &w->colors[color].joints, j->id );
		j->setIndex = O_SET_AWAKE;
	}
	for ( int i = 0; i < set->islands.count; ++i )
	{
		oIsland* island = w->islands + set->islands.data[i];
		island->setIndex = O_SET_AWAKE;
		island->localIndex = w->awakeIslands.count;
		oia_push( &w->awakeIslands, island->islandId );
	}
	destroy_solver_set( w, setIndex );
}

/* reference src/solver_set.c:162-451 */
void o_try_sleep_island( oWorld* w, int islandId )
{
	oIsland* island = w->islands + islandId;
	if ( island->constraintRemoveCount > 0 )
		return;

	int sleepSetId = o_create_sleeping_set( w );
	oSolverSet* sleepSet = w->sets + sleepSetId;

	/* bodies, and the non-touching contacts whose other body already sleeps */
	for ( int bodyId = island->headBody; bodyId != O_NULL; )
	{
		oBody* body = w->bodies + bodyId;
		int awakeIndex = body->awakeIndex;
		int sleepIndex = sleepSet->bodies.count;
		oia_push( &sleepSet->bodies, bodyId );
		int moved = oia_remove_swap( &w->awake, awakeIndex );
		if ( moved != O_NULL )
			w->bodies[w->awake.data[awakeIndex]].awakeIndex = awakeIndex;
		body->setIndex = sleepSetId;
		body->awakeIndex = O_NULL;
		body->setLocal = sleepIndex;

		int contactKey = body->headContactKey;
		while ( contactKey != O_NULL )
		{
			int edgeIndex = contactKey & 1;
			oContact* c = w->contacts + ( contactKey >> 1 );
			contactKey = c->edges[edgeIndex].nextKey;
			if ( c->setIndex == O_SET_DISABLED )
				continue;
			if ( c->colorIndex != O_NULL )
				continue;
			oBody* other = w->bodies + c->edges[edgeIndex ^ 1].bodyId;
			if ( other->setIndex == O_SET_AWAKE )
				continue;
			int localIndex = c->localIndex;
			c->setIndex = O_SET_DISABLED;
			c->localIndex = w->disabledContacts.count;
			oia_push( &w->disabledContacts, c->id );
			int movedContact = oia_remove_swap( &w->nonTouching, localIndex );
			if ( movedContact != O_NULL )
				w->contacts[w->nonTouching.data[localIndex]].localIndex = localIndex;
		}
		bodyId = body->islandNext;
	}

	/* touching contacts leave the graph */
	for ( int contactId = island->headContact; contactId != O_NULL; )
	{
		oContact* c = w->contacts + contactId;
		int colorIndex = c->colorIndex;
		oColor* color = w->colors + colorIndex;
		if ( colorIndex != O_OVERFLOW )
		{
			obits_clear( &color->bodySet, c->edges[0].bodyId );
			obits_clear( &color->bodySet, c->edges[1].bodyId );
		}
		int awakeContactIndex = c->localIndex;
		int sleepContactIndex = sleepSet->contacts.count;
		oia_push( &sleepSet->contacts, contactId );
		int moved = oia_remove_swap( &color->contacts, awakeContactIndex );
		if ( moved != O_NULL )
			w->contacts[color->contacts.data[awakeContactIndex]].localIndex = awakeContactIndex;
		c->setIndex = sleepSetId;
		c->colorIndex = O_NULL;
		c->localIndex = sleepContactIndex;
		contactId = c->islandNext;
	}

	/* joints leave the graph */
	for ( int jointId = island->headJoint; jointId != O_NULL; )
	{
		oJoint* j = w->joints + jointId;
		int colorIndex = j->colorIndex;
		int localIndex = j->localIndex;
		oColor* color = w->colors + colorIndex;
		if ( colorIndex != O_OVERFLOW )
		{
			obits_clear( &color->bodySet, j->edges[0].bodyId );
			obits_clear( &color->bodySet, j->edges[1].bodyId );
		}
		int sleepJointIndex = sleepSet->joints.count;
		oia_push( &sleepSet->joints, jointId );
		int moved = oia_remove_swap( &color->joints, localIndex );
		if ( moved != O_NULL )
			w->joints[color->joints.data[localIndex]].localIndex = localIndex;
		j->setIndex = sleepSetId;
		j->colorIndex = O_NULL;
		j->localIndex = sleepJointIndex;
		jointId = j->islandNext;
	}

	/* the island itself */
	{
		int islandIndex = island->localIndex;
		oia_push( &sleepSet->islands, islandId );
		int moved = oia_remove_swap( &w->awakeIslands, islandIndex );
		if ( moved != O_NULL )
			w->islands[w->awakeIslands.data[islandIndex]].localIndex = islandIndex;
		island->setIndex = sleepSetId;
		island->localIndex = 0;
	}
}

/* reference src/solver_set.c:456-554 */
void o_merge_solver_sets( oWorld* w, int setId1, int setId2 )
{
	oSolverSet* set1 = w->sets + setId1;
	oSolverSet* set2 = w->sets + setId2;
	if ( set1->bodies.count < set2->bodies.count )
	{
		oSolverSet* t = set1;
		set1 = set2;
		set2 = t;
		int ti = setId1;
		setId1 = setId2;
		setId2 = ti;
	}
	for ( int i = 0; i < set2->bodies.count; ++i )
	{
		oBody* body = w->bodies + set2->bodies.data[i];
		body->setIndex = setId1;
		body->setLocal = set1->bodies.count;
		oia_push( &set1->bodies, body->id );
	}
	for ( int i = 0; i < set2->contacts.count; ++i )
	{
		oContact* c = w->contacts + set2->contacts.data[i];
		c->setIndex = setId1;
		c->localIndex = set1->contacts.count;
		oia_push( &set1->contacts, c->id );
	}
	for ( int i = 0; i < set2->joints.count; ++i )
	{
		oJoint* j = w->joints + set2->joints.data[i];
		j->setIndex = setId1;
		j->localIndex = set1->joints.count;
		oia_push( &set1->joints, j->id );
	}
	for ( int i = 0; i < set2->islands.count; ++i )
	{
		oIsland* island = w->islands + set2->islands.data[i];
		island->setIndex = setId1;
		island->localIndex = set1->islands.count;
		oia_push( &set1->islands, island->islandId );
	}
	destroy_solver_set( w, setId2 );
}

/* reference src/body.c:325-333 */
bool o_wake_body( oWorld* w, oBody* b )
{
	if ( b->setIndex >= O_SET_FIRST_SLEEPING )
	{
		o_wake_solver_set( w, b->setIndex );
		return true;
	}
	return false;
}
