/*
 * adjoint.cu -- reverse-mode gradient of recorded steps (b2World_StepBackward).
 *
 * Forward: while a world's tape is active, every step records its solver inputs before
 * the solver stage runs (k_tape_record): body states at the step start and the
 * coloured rows with the manifolds the narrowphase produced (warm-start impulses
 * included).
 *
 * Backward (k_adjoint, one warp per world, steps in reverse): each step is first
 * replayed forward from its record -- the same b2g_solve.h arithmetic in the same
 * order, so the replay is bit-identical -- keeping per-substep body snapshots and, for
 * every row and phase, the velocities and impulses the row started from; the contact
 * geometry is recomputed with dual numbers (b2g_dual.h) for its Jacobian.  Then the
 * step is differentiated backwards: finalisation, restitution colours in reverse
 * order, and per substep in reverse: relax colours reversed, position integration,
 * solve colours reversed, warm-start colours reversed, velocity integration; then the
 * row preparation and the narrowphase Jacobian.  Within a colour no two rows share a
 * body, so a colour's row adjoints run in parallel lanes without conflicts.  The
 * adjoint of the warm-start impulses goes to the previous step's stored impulses
 * through the narrowphase's feature-id matching (reference src/contact.c:555-568).
 *
 * Differentiated: body centres, angles, linear and angular velocities, and contact
 * friction (mixed per shape as sqrt(muA * muB), reference src/contact.c:42-45).  The
 * discrete choices of a step (pairs, colours, manifold features, active clamps) are
 * those of the recorded forward step.  Polygon, capsule, segment and circle shapes, and
 * rows in the graph colours and in the overflow colour; joints and chain links are
 * reported as unsupported.
 *
 * Reference arithmetic being differentiated: src/solver.c:34-93, :146-163, :205-223;
 * src/contact_solver.c:597-1293; src/manifold.c:276-700.
 */
#include "b2g_dual.h"
#include "b2g_stages.h"

#include <cuda_runtime.h>

/* ------------------------------------------------------------------ recording */
__global__ void k_tape_record( b2gDevWorld W, float4* bodies, int bodyCount, b2gTapeRow* rows, int rowCount )
{
	tape_record_one( W, bodies, bodyCount, rows, rowCount, blockIdx.x * blockDim.x + threadIdx.x );
}

extern "C" int b2gd_tape_record( b2gDevWorld* w, void* bodyDst, int bodies, void* rowDst, int rows )
{
	int n = bodies > rows ? bodies : rows;
	if ( n <= 0 )
		return 0;
	k_tape_record<<<( n + 255 ) / 256, 256, 0, (cudaStream_t)w->stream>>>( *w, (float4*)bodyDst, bodies, (b2gTapeRow*)rowDst, rows );
	return (int)cudaGetLastError();
}

/* ------------------------------------------------------------------ scratch layout */
/* Per body: adjoint (12), replay state (8), step start (12), velocity terms (8).
 * Per body and snapshot: 8.  Per row: Row (64), adjoint (24), Jacobian (72), and 12
 * per phase.  Per contact id: impulse adjoint (4) + stamp, previous-step row + stamp. */
#define ADJ_BODY 12
#define ADJ_STATE 8
#define ADJ_START 12
#define ADJ_TERMS 8
#define ADJ_SNAP 8
#define ADJ_ROW 64
#define ADJ_RADJ 24
#define ADJ_JAC 72
#define ADJ_PHASE 12
#define ADJ_MAX_SUBSTEPS 16

static_assert( sizeof( Row ) <= ADJ_ROW * 4, "row record must fit its scratch slot" );

struct AdjLayout
{
	float* bodyAdj;
	float* state;
	float* start;
	float* terms;
	float* snap;
	float* rows;
	float* radj;
	float* jac;
	float* phase;
	float* lam;	 /* 4 per contact id */
	int* lamStamp;
	int* prevRow;
	int* prevStamp;
};

static __host__ __device__ size_t adj_layout( AdjLayout* L, float* base, int N, int R, int C, int S )
{
	size_t o = 0;
	float* b = base;
	auto take = [&]( size_t n ) {
		float* p = b ? b + o : nullptr;
		o += ( n + 3 ) & ~(size_t)3;
		return p;
	};
	AdjLayout l;
	l.bodyAdj = take( (size_t)N * ADJ_BODY );
	l.state = take( (size_t)N * ADJ_STATE );
	l.start = take( (size_t)N * ADJ_START );
	l.terms = take( (size_t)N * ADJ_TERMS );
	l.snap = take( (size_t)( 2 * S + 1 ) * N * ADJ_SNAP );
	l.rows = take( (size_t)R * ADJ_ROW );
	l.radj = take( (size_t)R * ADJ_RADJ );
	l.jac = take( (size_t)R * ADJ_JAC );
	l.phase = take( (size_t)( 3 * S + 1 ) * R * ADJ_PHASE );
	l.lam = take( (size_t)C * 4 );
	l.lamStamp = (int*)take( (size_t)C );
	l.prevRow = (int*)take( (size_t)C );
	l.prevStamp = (int*)take( (size_t)C );
	if ( L )
		*L = l;
	return o;
}

extern "C" size_t b2gd_adjoint_scratch( int bodies, int maxRows, int contactCap, int subSteps )
{
	int S = subSteps < 1 ? 1 : subSteps;
	return adj_layout( nullptr, nullptr, bodies, maxRows < 1 ? 1 : maxRows, contactCap < 1 ? 1 : contactCap, S );
}

/* ------------------------------------------------------------------ helpers */
struct BodyV
{
	float vx, vy, w;
};

struct RowAdj
{
	float n[2];
	float rA[2][2];
	float rB[2][2];
	float base[2];
	float nMass[2];
	float tMass[2];
	float relVel[2];
	float mu;
	float ni[2];
	float ti[2];
	float pad;
};
static_assert( sizeof( RowAdj ) == ADJ_RADJ * 4, "row adjoint layout" );

__device__ __forceinline__ BodyV bv_of( const DevState& s )
{
	BodyV v;
	v.vx = s.v.x;
	v.vy = s.v.y;
	v.w = s.w;
	return v;
}

/* VJP of the impulse application of the 8-lane path (lane_apply / warm_lane):
 * a.v -= mA P, a.w -= iA cross(rA, P), b.v += mB P, b.w += iB cross(rB, P). */
__device__ __forceinline__ b2gVec apply_vjp( b2gVec P, b2gVec rA, b2gVec rB, const Row& r, const BodyV& aA, const BodyV& aB, float* rAbar,
											 float* rBbar )
{
	b2gVec Pb;
	Pb.x = r.mB * aB.vx - r.mA * aA.vx + r.iB * aB.w * ( -rB.y ) - r.iA * aA.w * ( -rA.y );
	Pb.y = r.mB * aB.vy - r.mA * aA.vy + r.iB * aB.w * rB.x - r.iA * aA.w * rA.x;
	rAbar[0] += -r.iA * aA.w * P.y;
	rAbar[1] += r.iA * aA.w * P.x;
	rBbar[0] += r.iB * aB.w * P.y;
	rBbar[1] += -r.iB * aB.w * P.x;
	return Pb;
}

/* VJP of the lane relative velocity dv = (vB + wB x rB) - (vA + wA x rA). */
__device__ __forceinline__ void dv_vjp( b2gVec g, b2gVec rA, b2gVec rB, float wA, float wB, BodyV& aA, BodyV& aB, float* rAbar, float* rBbar )
{
	aB.vx += g.x;
	aB.vy += g.y;
	aA.vx -= g.x;
	aA.vy -= g.y;
	aB.w += -rB.y * g.x + rB.x * g.y;
	aA.w -= -rA.y * g.x + rA.x * g.y;
	rBbar[0] += wB * g.y;
	rBbar[1] += -wB * g.x;
	rAbar[0] -= wA * g.y;
	rAbar[1] -= -wA * g.x;
}

__device__ __forceinline__ b2gVec lane_dv( const DevState& a, const DevState& b, b2gVec aA, b2gVec aB )
{
	float dvx = ( b.v.x - b.w * aB.y ) - ( a.v.x - a.w * aA.y );
	float dvy = ( b.v.y + b.w * aB.x ) - ( a.v.y + a.w * aA.x );
	return gv( dvx, dvy );
}

/* ------------------------------------------------------------------ row VJPs */
/* Warm start (linear in the impulses). */
__device__ void warm_vjp( const Row& r, const BodyV& aA, const BodyV& aB, RowAdj& ra )
{
	b2gVec n = r.n;
	b2gVec t = gv( n.y, 0.0f - n.x );
	for ( int j = 0; j < 2; ++j )
	{
		b2gVec P = gv( r.ni[j] * n.x + r.ti[j] * t.x, r.ni[j] * n.y + r.ti[j] * t.y );
		b2gVec Pb = apply_vjp( P, r.rA[j], r.rB[j], r, aA, aB, ra.rA[j], ra.rB[j] );
		ra.ni[j] += Pb.x * n.x + Pb.y * n.y;
		ra.ti[j] += Pb.x * t.x + Pb.y * t.y;
		ra.n[0] += r.ni[j] * Pb.x - r.ti[j] * Pb.y;
		ra.n[1] += r.ni[j] * Pb.y + r.ti[j] * Pb.x;
	}
}

/* Solve / relax.  r holds the impulses before the row ran; a, b the states before it
 * (velocities) and the substep's position deltas.  On entry aA, aB are the adjoints of
 * the velocities after the row; on exit, before it.  dpA.. receive the position-delta
 * adjoints.  scalar: an overflow row, whose speculative points (s > 0) take the rigid
 * mass and no impulse scaling where the 8-lane rows keep the soft ones (reference
 * src/contact_solver.c:266-279 against :905-925). */
__device__ void solve_vjp( Row r, DevState a, DevState b, bool useBias, const b2gStepConst& sc, BodyV& aA, BodyV& aB, RowAdj& ra,
						   float* dpA, float* dqA, float* dpB, float* dqB, bool scalar = false )
{
	float biasRate = useBias ? r.biasRate : 0.0f;
	float massScale = useBias ? r.massScale : 1.0f;
	float impulseScale = useBias ? r.impulseScale : 0.0f;
	float minBias = -sc.pushout;
	b2gVec n = r.n;
	b2gVec t = gv( n.y, 0.0f - n.x );
	b2gVec dp = gv( b.dp.x - a.dp.x, b.dp.y - a.dp.y );

	/* forward replay with snapshots before each of the four point updates */
	DevState sa[4], sb[4];
	float ni0[2] = { r.ni[0], r.ni[1] };
	float ti0[2] = { r.ti[0], r.ti[1] };
	float s_[2], dbds[2], xN[2], ms_[2], is_[2];
	for ( int j = 0; j < 2; ++j )
	{
		sa[j] = a;
		sb[j] = b;
		b2gVec aA_ = r.rA[j], aB_ = r.rB[j];
		b2gVec rsA = gv( a.dq.c * aA_.x - a.dq.s * aA_.y, a.dq.s * aA_.x + a.dq.c * aA_.y );
		b2gVec rsB = gv( b.dq.c * aB_.x - b.dq.s * aB_.y, b.dq.s * aB_.x + b.dq.c * aB_.y );
		b2gVec ds = gv( dp.x + ( rsB.x - rsA.x ), dp.y + ( rsB.y - rsA.y ) );
		float s = ( n.x * ds.x + n.y * ds.y ) + r.base[j];
		float bias;
		if ( s > 0.0f )
		{
			bias = s * sc.inv_h;
			dbds[j] = sc.inv_h;
		}
		else
		{
			float soft = biasRate * s;
			bias = gmax( soft, minBias );
			dbds[j] = soft > minBias ? biasRate : 0.0f;
		}
		s_[j] = s;
		ms_[j] = scalar && s > 0.0f ? 1.0f : massScale;
		is_[j] = scalar && s > 0.0f ? 0.0f : impulseScale;
		b2gVec dv = lane_dv( a, b, aA_, aB_ );
		float vn = dv.x * n.x + dv.y * n.y;
		float negImpulse = r.nMass[j] * ( ms_[j] * ( vn + bias ) ) + is_[j] * r.ni[j];
		float x = r.ni[j] - negImpulse;
		xN[j] = x;
		float newImpulse = gmax( x, 0.0f );
		float impulse = newImpulse - r.ni[j];
		r.ni[j] = newImpulse;
		lane_apply( a, b, r, aA_, aB_, impulse * n.x, impulse * n.y );
	}
	float xT[2], maxF[2];
	int clampT[2]; /* 0 interior, 1 upper, -1 lower */
	for ( int j = 0; j < 2; ++j )
	{
		sa[2 + j] = a;
		sb[2 + j] = b;
		b2gVec aA_ = r.rA[j], aB_ = r.rB[j];
		b2gVec dv = lane_dv( a, b, aA_, aB_ );
		float vt = dv.x * t.x + dv.y * t.y;
		float negImpulse = r.tMass[j] * vt;
		float maxFriction = r.friction * r.ni[j];
		float x = r.ti[j] - negImpulse;
		float lo = 0.0f - maxFriction;
		float mn = x < maxFriction ? x : maxFriction;
		float newImpulse = lo > mn ? lo : mn;
		clampT[j] = lo > mn ? -1 : ( x < maxFriction ? 0 : 1 );
		xT[j] = x;
		maxF[j] = maxFriction;
		float impulse = newImpulse - r.ti[j];
		r.ti[j] = newImpulse;
		lane_apply( a, b, r, aA_, aB_, impulse * t.x, impulse * t.y );
	}

	/* tangent points in reverse */
	for ( int j = 1; j >= 0; --j )
	{
		const DevState& A = sa[2 + j];
		const DevState& B = sb[2 + j];
		float newImpulse = clampT[j] < 0 ? -maxF[j] : ( clampT[j] == 0 ? xT[j] : maxF[j] );
		float impulse = newImpulse - ti0[j];
		b2gVec P = gv( impulse * t.x, impulse * t.y );
		b2gVec Pb = apply_vjp( P, r.rA[j], r.rB[j], r, aA, aB, ra.rA[j], ra.rB[j] );
		float impb = Pb.x * t.x + Pb.y * t.y;
		ra.n[0] += -( impulse * Pb.y );
		ra.n[1] += impulse * Pb.x;
		float newb = ra.ti[j] + impb;
		float tib = -impb;
		float xb = 0.0f, maxFb = 0.0f;
		if ( clampT[j] < 0 )
			maxFb = -newb;
		else if ( clampT[j] == 0 )
			xb = newb;
		else
			maxFb = newb;
		ra.mu += maxFb * r.ni[j];
		ra.ni[j] += maxFb * r.friction;
		tib += xb;
		float negb = -xb;
		b2gVec dv = lane_dv( A, B, r.rA[j], r.rB[j] );
		float vt = dv.x * t.x + dv.y * t.y;
		ra.tMass[j] += negb * vt;
		float vtb = negb * r.tMass[j];
		/* vt = dv . t, t = ( n.y, -n.x ) */
		ra.n[0] += -( vtb * dv.y );
		ra.n[1] += vtb * dv.x;
		dv_vjp( gv( vtb * t.x, vtb * t.y ), r.rA[j], r.rB[j], A.w, B.w, aA, aB, ra.rA[j], ra.rB[j] );
		ra.ti[j] = tib;
	}
	/* normal points in reverse */
	for ( int j = 1; j >= 0; --j )
	{
		const DevState& A = sa[j];
		const DevState& B = sb[j];
		float newImpulse = gmax( xN[j], 0.0f );
		float impulse = newImpulse - ni0[j];
		b2gVec P = gv( impulse * n.x, impulse * n.y );
		b2gVec Pb = apply_vjp( P, r.rA[j], r.rB[j], r, aA, aB, ra.rA[j], ra.rB[j] );
		float impb = Pb.x * n.x + Pb.y * n.y;
		ra.n[0] += impulse * Pb.x;
		ra.n[1] += impulse * Pb.y;
		float newb = ra.ni[j] + impb;
		float nib = -impb;
		float xb = xN[j] > 0.0f ? newb : 0.0f;
		nib += xb;
		float negb = -xb;
		b2gVec dv = lane_dv( A, B, r.rA[j], r.rB[j] );
		float vn = dv.x * n.x + dv.y * n.y;
		/* negImpulse = nMass * ( massScale * ( vn + bias ) ) + impulseScale * ni */
		float s = s_[j];
		float bias = s > 0.0f ? s * sc.inv_h : gmax( biasRate * s, minBias );
		ra.nMass[j] += negb * ( ms_[j] * ( vn + bias ) );
		float vnb = negb * r.nMass[j] * ms_[j];
		nib += negb * is_[j];
		float sb_ = vnb * dbds[j];
		ra.n[0] += vnb * dv.x;
		ra.n[1] += vnb * dv.y;
		dv_vjp( gv( vnb * n.x, vnb * n.y ), r.rA[j], r.rB[j], A.w, B.w, aA, aB, ra.rA[j], ra.rB[j] );
		/* s = n . ( dp + rotate( dqB, rB ) - rotate( dqA, rA ) ) + base */
		b2gVec aA_ = r.rA[j], aB_ = r.rB[j];
		b2gVec rsA = gv( A.dq.c * aA_.x - A.dq.s * aA_.y, A.dq.s * aA_.x + A.dq.c * aA_.y );
		b2gVec rsB = gv( B.dq.c * aB_.x - B.dq.s * aB_.y, B.dq.s * aB_.x + B.dq.c * aB_.y );
		b2gVec ds = gv( dp.x + ( rsB.x - rsA.x ), dp.y + ( rsB.y - rsA.y ) );
		ra.n[0] += sb_ * ds.x;
		ra.n[1] += sb_ * ds.y;
		ra.base[j] += sb_;
		b2gVec dsb = gv( sb_ * n.x, sb_ * n.y );
		dpB[0] += dsb.x;
		dpB[1] += dsb.y;
		dpA[0] -= dsb.x;
		dpA[1] -= dsb.y;
		/* rotate( q, v ): d/dq.c = v, d/dq.s = ( -v.y, v.x ); d/dv = rotate^T */
		dqB[0] += dsb.x * aB_.x + dsb.y * aB_.y;
		dqB[1] += -dsb.x * aB_.y + dsb.y * aB_.x;
		dqA[0] -= dsb.x * aA_.x + dsb.y * aA_.y;
		dqA[1] -= -dsb.x * aA_.y + dsb.y * aA_.x;
		ra.rB[j][0] += B.dq.c * dsb.x + B.dq.s * dsb.y;
		ra.rB[j][1] += -B.dq.s * dsb.x + B.dq.c * dsb.y;
		ra.rA[j][0] -= A.dq.c * dsb.x + A.dq.s * dsb.y;
		ra.rA[j][1] -= -A.dq.s * dsb.x + A.dq.c * dsb.y;
		ra.ni[j] = nib;
	}
}

/* Restitution (8-lane path). */
__device__ void restitution_vjp( Row r, DevState a, DevState b, const b2gStepConst& sc, BodyV& aA, BodyV& aB, RowAdj& ra )
{
	b2gVec n = r.n;
	DevState sa[2], sb[2];
	float xN[2], ni0[2] = { r.ni[0], r.ni[1] }, mass[2];
	for ( int j = 0; j < 2; ++j )
	{
		sa[j] = a;
		sb[j] = b;
		bool skip = ( r.relVel[j] + sc.restitutionThreshold > 0.0f ) || ( r.maxNi[j] == 0.0f );
		mass[j] = skip ? 0.0f : r.nMass[j];
		b2gVec dv = lane_dv( a, b, r.rA[j], r.rB[j] );
		float vn = dv.x * n.x + dv.y * n.y;
		float negImpulse = mass[j] * ( vn + r.restitution * r.relVel[j] );
		float x = r.ni[j] - negImpulse;
		xN[j] = x;
		float newImpulse = gmax( x, 0.0f );
		float impulse = newImpulse - r.ni[j];
		r.ni[j] = newImpulse;
		lane_apply( a, b, r, r.rA[j], r.rB[j], impulse * n.x, impulse * n.y );
	}
	for ( int j = 1; j >= 0; --j )
	{
		const DevState& A = sa[j];
		const DevState& B = sb[j];
		float newImpulse = gmax( xN[j], 0.0f );
		float impulse = newImpulse - ni0[j];
		b2gVec P = gv( impulse * n.x, impulse * n.y );
		b2gVec Pb = apply_vjp( P, r.rA[j], r.rB[j], r, aA, aB, ra.rA[j], ra.rB[j] );
		float impb = Pb.x * n.x + Pb.y * n.y;
		ra.n[0] += impulse * Pb.x;
		ra.n[1] += impulse * Pb.y;
		float newb = ra.ni[j] + impb;
		float nib = -impb;
		float xb = xN[j] > 0.0f ? newb : 0.0f;
		nib += xb;
		float negb = -xb;
		b2gVec dv = lane_dv( A, B, r.rA[j], r.rB[j] );
		float vn = dv.x * n.x + dv.y * n.y;
		if ( mass[j] != 0.0f )
			ra.nMass[j] += negb * ( vn + r.restitution * r.relVel[j] );
		float inner = negb * mass[j];
		ra.relVel[j] += inner * r.restitution;
		ra.n[0] += inner * dv.x;
		ra.n[1] += inner * dv.y;
		dv_vjp( gv( inner * n.x, inner * n.y ), r.rA[j], r.rB[j], A.w, B.w, aA, aB, ra.rA[j], ra.rB[j] );
		ra.ni[j] = nib;
	}
}

/* ------------------------------------------------------------------ body VJPs */
/* Body adjoint layout (12 floats): c.x c.y q.c q.s | v.x v.y w | dp.x dp.y | dq.c dq.s | - */

/* integrate_velocity: v' = cap( lvd + ld v ), w' = cap( avd + ad w ) */
__device__ void iv_vjp( const float* pre, float4 term, float ad, const b2gStepConst& sc, float* g )
{
	float maxLin = B2G_MAX_TRANSLATION * sc.inv_dt;
	float maxAng = B2G_MAX_ROTATION * sc.inv_dt;
	b2gVec v = gmuladd( gv( term.x, term.y ), term.w, gv( pre[0], pre[1] ) );
	float w = term.z + ad * pre[2];
	float gx = g[4], gy = g[5], gw = g[6];
	if ( gdot( v, v ) > maxLin * maxLin )
	{
		float L = glen( v );
		float k = maxLin / L;
		b2gVec u = gv( v.x / L, v.y / L );
		float d = gx * u.x + gy * u.y;
		gx = k * ( gx - d * u.x );
		gy = k * ( gy - d * u.y );
	}
	if ( w * w > maxAng * maxAng )
		gw = 0.0f;
	g[4] = term.w * gx;
	g[5] = term.w * gy;
	g[6] = ad * gw;
}

/* integrate_position: dq' = normalize( dq + h w perp( dq ) ), dp' = dp + h v */
__device__ void ip_vjp( const float* pre, float h, float* g )
{
	float dqc = pre[6], dqs = pre[7];
	float da = h * pre[2];
	float q2c = dqc - da * dqs, q2s = dqs + da * dqc;
	float mag = sqrtf( q2s * q2s + q2c * q2c );
	float inv = mag > 0.0f ? 1.0f / mag : 0.0f;
	float nc = q2c * inv, ns = q2s * inv;
	float d = nc * g[9] + ns * g[10];
	float g2c = ( g[9] - nc * d ) * inv, g2s = ( g[10] - ns * d ) * inv;
	g[9] = g2c + da * g2s;
	g[10] = -da * g2c + g2s;
	g[6] += h * ( -dqs * g2c + dqc * g2s );
	g[4] += h * g[7];
	g[5] += h * g[8];
}

/* finalisation: c' = c + dp, q' = normalize( dq q ) (reference src/solver.c:205-223) */
__device__ void finalize_vjp( float qc, float qs, float dqc, float dqs, float* g )
{
	float us = dqs * qc + dqc * qs;
	float uc = dqc * qc - dqs * qs;
	float mag = sqrtf( us * us + uc * uc );
	float inv = mag > 0.0f ? 1.0f / mag : 0.0f;
	float nc = uc * inv, ns = us * inv;
	float d = nc * g[2] + ns * g[3];
	float guc = ( g[2] - nc * d ) * inv, gus = ( g[3] - ns * d ) * inv;
	g[9] = guc * qc + gus * qs;
	g[10] = -guc * qs + gus * qc;
	g[2] = guc * dqc + gus * dqs;
	g[3] = -guc * dqs + gus * dqc;
	g[7] = g[0];
	g[8] = g[1];
}

/* ------------------------------------------------------------------ prepare VJP */
/* Adjoint of the row preparation (reference src/contact_solver.c:597-808) with
 * respect to the manifold (normal, centre-relative anchors, separations), the bodies'
 * step-start velocities and the warm-start impulses.  mAdj: n(2), then per point
 * anchorA(2) anchorB(2) separation. */
__device__ void prepare_vjp( const Row& r, const DevState& sA, const DevState& sB, const RowAdj& ra, float warm, float* mAdj, BodyV& aA,
							 BodyV& aB, float* lamIn )
{
	b2gVec n = r.n;
	b2gVec t = gright( n );
	float nb[2] = { ra.n[0], ra.n[1] };
	float tb[2] = { 0.0f, 0.0f };
	for ( int i = 0; i < 12; ++i )
		mAdj[i] = 0.0f;
	for ( int i = 0; i < 4; ++i )
		lamIn[i] = 0.0f;
	for ( int j = 0; j < r.count; ++j )
	{
		b2gVec rA = r.rA[j], rB = r.rB[j];
		float rAb[2] = { ra.rA[j][0], ra.rA[j][1] };
		float rBb[2] = { ra.rB[j][0], ra.rB[j][1] };
		/* base = separation - ( rB - rA ) . n */
		float gb = ra.base[j];
		float sepb = gb;
		rBb[0] -= gb * n.x;
		rBb[1] -= gb * n.y;
		rAb[0] += gb * n.x;
		rAb[1] += gb * n.y;
		nb[0] -= gb * ( rB.x - rA.x );
		nb[1] -= gb * ( rB.y - rA.y );
		/* normal and tangent mass: 1 / ( mA + mB + iA rn_A^2 + iB rn_B^2 ) */
		if ( r.nMass[j] > 0.0f )
		{
			float rnA = gcross( rA, n ), rnB = gcross( rB, n );
			float gk = -ra.nMass[j] * r.nMass[j] * r.nMass[j];
			float grA = gk * 2.0f * r.iA * rnA, grB = gk * 2.0f * r.iB * rnB;
			rAb[0] += grA * n.y;
			rAb[1] += -grA * n.x;
			nb[0] += -grA * rA.y;
			nb[1] += grA * rA.x;
			rBb[0] += grB * n.y;
			rBb[1] += -grB * n.x;
			nb[0] += -grB * rB.y;
			nb[1] += grB * rB.x;
		}
		if ( r.tMass[j] > 0.0f )
		{
			float rtA = gcross( rA, t ), rtB = gcross( rB, t );
			float gk = -ra.tMass[j] * r.tMass[j] * r.tMass[j];
			float grA = gk * 2.0f * r.iA * rtA, grB = gk * 2.0f * r.iB * rtB;
			rAb[0] += grA * t.y;
			rAb[1] += -grA * t.x;
			tb[0] += -grA * rA.y;
			tb[1] += grA * rA.x;
			rBb[0] += grB * t.y;
			rBb[1] += -grB * t.x;
			tb[0] += -grB * rB.y;
			tb[1] += grB * rB.x;
		}
		/* relative normal velocity at the step start */
		float gr = ra.relVel[j];
		b2gVec dv = gsub( gadd( sB.v, gcross_sv( sB.w, rB ) ), gadd( sA.v, gcross_sv( sA.w, rA ) ) );
		nb[0] += gr * dv.x;
		nb[1] += gr * dv.y;
		dv_vjp( gv( gr * n.x, gr * n.y ), rA, rB, sA.w, sB.w, aA, aB, rAb, rBb );
		lamIn[j] = warm * ra.ni[j];
		lamIn[2 + j] = warm * ra.ti[j];
		mAdj[2 + 5 * j + 0] = rAb[0];
		mAdj[2 + 5 * j + 1] = rAb[1];
		mAdj[2 + 5 * j + 2] = rBb[0];
		mAdj[2 + 5 * j + 3] = rBb[1];
		mAdj[2 + 5 * j + 4] = sepb;
	}
	/* t = ( n.y, -n.x ) */
	nb[0] += -tb[1];
	nb[1] += tb[0];
	mAdj[0] = nb[0];
	mAdj[1] = nb[1];
}

/* ------------------------------------------------------------------ narrowphase Jacobian */
/* Recomputes the manifold of a polygon pair with derivatives in the six directions
 * ( cA.x, cA.y, angleA, cB.x, cB.y, angleB ); writes the 12 x 6 Jacobian of
 * ( normal, per point anchorA anchorB separation ), anchors relative to the centres.
 * Returns false when the replay does not reproduce the recorded manifold. */
__device__ bool manifold_jacobian( const b2gShapeGeo& gA, const b2gShapeGeo& gB, const float* startA, const float* startB, bool dynA, bool dynB,
								   const b2gManifold& rec, float* jac )
{
	typedef Dual<6> D;
	DXf<6> xf[2];
	const float* st[2] = { startA, startB };
	bool dyn[2] = { dynA, dynB };
	DRot<6> q[2];
	for ( int k = 0; k < 2; ++k )
	{
		/* start record: c.x c.y q.c q.s lc.x lc.y p.x p.y */
		float qc = st[k][2], qs = st[k][3], lcx = st[k][4], lcy = st[k][5];
		D px = dc<6>( st[k][6] ), py = dc<6>( st[k][7] );
		D c = dc<6>( qc ), s = dc<6>( qs );
		if ( dyn[k] )
		{
			int o = 3 * k;
			px.d[o + 0] = 1.0f;
			py.d[o + 1] = 1.0f;
			/* p = c - rotate( q, lc ) */
			px.d[o + 2] = qs * lcx + qc * lcy;
			py.d[o + 2] = -qc * lcx + qs * lcy;
			c.d[o + 2] = -qs;
			s.d[o + 2] = qc;
		}
		xf[k].p = dv( px, py );
		xf[k].q.c = c;
		xf[k].q.s = s;
		q[k] = xf[k].q;
	}
	/* the narrowphase's dispatch (b2g_collide.h gcollide_shapes) for A not a chain link */
	DManifold<6> m;
	if ( gB.type == 0 )
	{
		if ( gA.type == 0 )
			dcollide_circles( m, gA.v[0], gA.radius, xf[0], gB.v[0], gB.radius, xf[1] );
		else if ( gA.type == 1 || gA.type == 2 )
			dcollide_capsule_circle( m, gA.v[0], gA.v[1], gA.type == 1 ? gA.radius : 0.0f, xf[0], gB.v[0], gB.radius, xf[1] );
		else
		{
			b2gPoly pa;
			gshape_poly( &pa, &gA );
			dcollide_polygon_circle( m, pa, xf[0], gB.v[0], gB.radius, xf[1] );
		}
	}
	else
	{
		b2gPoly pa, pb;
		gshape_poly( &pa, &gA );
		gshape_poly( &pb, &gB );
		dcollide_polygons( m, pa, xf[0], pb, xf[1] );
	}
	DVec<6> offA = drotate( q[0], dvc<6>( gv( startA[4], startA[5] ) ) );
	DVec<6> offB = drotate( q[1], dvc<6>( gv( startB[4], startB[5] ) ) );
	bool same = m.count == rec.count && m.normal.x.v == rec.normal.x && m.normal.y.v == rec.normal.y;
	for ( int i = 0; i < 12 * 6; ++i )
		jac[i] = 0.0f;
	for ( int d = 0; d < 6; ++d )
	{
		jac[0 * 6 + d] = m.normal.x.d[d];
		jac[1 * 6 + d] = m.normal.y.d[d];
	}
	for ( int j = 0; j < m.count && j < 2; ++j )
	{
		DVec<6> aA = dsub( m.pts[j].anchorA, offA );
		DVec<6> aB = dsub( m.pts[j].anchorB, offB );
		same = same && aA.x.v == rec.pts[j].anchorA.x && aA.y.v == rec.pts[j].anchorA.y && aB.x.v == rec.pts[j].anchorB.x &&
			   aB.y.v == rec.pts[j].anchorB.y && m.pts[j].separation.v == rec.pts[j].separation && m.pts[j].id == rec.pts[j].id;
		for ( int d = 0; d < 6; ++d )
		{
			jac[( 2 + 5 * j + 0 ) * 6 + d] = aA.x.d[d];
			jac[( 2 + 5 * j + 1 ) * 6 + d] = aA.y.d[d];
			jac[( 2 + 5 * j + 2 ) * 6 + d] = aB.x.d[d];
			jac[( 2 + 5 * j + 3 ) * 6 + d] = aB.y.d[d];
			jac[( 2 + 5 * j + 4 ) * 6 + d] = m.pts[j].separation.d[d];
		}
	}
	return same;
}

/* ------------------------------------------------------------------ the backward kernel */
#define ADJ_WARP 32

__device__ __forceinline__ DevState replay_state( const AdjLayout& L, int b )
{
	if ( b < 0 )
		return identity_state();
	const float* s = L.state + (size_t)b * ADJ_STATE;
	return state_of( make_float4( s[0], s[1], s[2], s[3] ), make_float4( s[4], s[5], s[6], s[7] ) );
}

__device__ __forceinline__ void replay_store_velocity( const AdjLayout& L, int b, const DevState& x )
{
	if ( b < 0 )
		return;
	float* s = L.state + (size_t)b * ADJ_STATE;
	s[0] = x.v.x;
	s[1] = x.v.y;
	s[2] = x.w;
}

__device__ __forceinline__ Row load_row_rec( const AdjLayout& L, int k ) { return *(const Row*)( L.rows + (size_t)k * ADJ_ROW ); }
__device__ __forceinline__ void store_row_rec( const AdjLayout& L, int k, const Row& r ) { *(Row*)( L.rows + (size_t)k * ADJ_ROW ) = r; }

/* One forward stage of the replay over the active colours (warm 0, solve 1, relax 2,
 * restitution 3), recording each row's starting velocities and impulses. */
/* The state a row starts from, kept on the phase tape for its reverse. */
__device__ __forceinline__ void tape_row_start( float* t, const Row& r, const DevState& A, const DevState& B )
{
	t[0] = A.v.x;
	t[1] = A.v.y;
	t[2] = A.w;
	t[3] = B.v.x;
	t[4] = B.v.y;
	t[5] = B.w;
	t[6] = r.ni[0];
	t[7] = r.ni[1];
	t[8] = r.ti[0];
	t[9] = r.ti[1];
	t[10] = r.maxNi[0];
	t[11] = r.maxNi[1];
}

__device__ void replay_stage( const AdjLayout& L, const b2gTapeStep& h, int R, int phase, int tapeIndex, const b2gStepConst& sc )
{
	float* tape = L.phase + (size_t)tapeIndex * R * ADJ_PHASE;
	/* the overflow colour first, one row after another with the scalar arithmetic
	 * (reference src/contact_solver.c:149-440) */
	if ( threadIdx.x == 0 )
	{
		for ( int k = h.colorStart[B2G_OVERFLOW]; k < h.colorStart[B2G_COLORS]; ++k )
		{
			Row r = load_row_rec( L, k );
			DevState A = replay_state( L, r.ia );
			DevState B = replay_state( L, r.ib );
			tape_row_start( tape + (size_t)k * ADJ_PHASE, r, A, B );
			bool changed = true;
			if ( phase == 0 )
				warm_scalar( r, A, B );
			else if ( phase == 3 )
				changed = restitution_scalar( r, A, B, sc.restitutionThreshold );
			else
				solve_scalar( r, A, B, phase == 1, sc.inv_h, sc.pushout );
			if ( changed )
			{
				replay_store_velocity( L, r.ia, A );
				replay_store_velocity( L, r.ib, B );
				store_row_rec( L, k, r );
			}
		}
	}
	__syncwarp();
	for ( int a = 0; a < h.activeCount; ++a )
	{
		int c = h.active[a];
		for ( int k = h.colorStart[c] + (int)threadIdx.x; k < h.colorStart[c + 1]; k += ADJ_WARP )
		{
			Row r = load_row_rec( L, k );
			DevState A = replay_state( L, r.ia );
			DevState B = replay_state( L, r.ib );
			tape_row_start( tape + (size_t)k * ADJ_PHASE, r, A, B );
			if ( phase == 0 )
				warm_lane( r, A, B );
			else if ( phase == 3 )
				restitution_lane( r, A, B, sc.restitutionThreshold );
			else
				solve_lane( r, A, B, phase == 1, sc.inv_h, sc.pushout );
			replay_store_velocity( L, r.ia, A );
			replay_store_velocity( L, r.ib, B );
			store_row_rec( L, k, r );
		}
		__syncwarp();
	}
}

/* Reverse of one row of a stage (its velocity, impulse and position-delta adjoints).
 * The scalar overflow rows share the lane rows' derivatives: the arithmetic is the same
 * up to operand grouping, a point past the manifold's count is a zero point of the lane
 * layout, and a restitution-free overflow row is skipped as the forward skipped it. */
__device__ void reverse_row( const AdjLayout& L, const float* tape, int k, int phase, const float* snap, const b2gStepConst& sc,
							 bool scalar )
{
	Row r = load_row_rec( L, k );
	if ( scalar && phase == 3 && r.restitution == 0.0f )
		return;
	const float* t = tape + (size_t)k * ADJ_PHASE;
	r.ni[0] = t[6];
	r.ni[1] = t[7];
	r.ti[0] = t[8];
	r.ti[1] = t[9];
	r.maxNi[0] = t[10];
	r.maxNi[1] = t[11];
	DevState A = identity_state(), B = identity_state();
	A.v = gv( t[0], t[1] );
	A.w = t[2];
	B.v = gv( t[3], t[4] );
	B.w = t[5];
	if ( snap && r.ia >= 0 )
	{
		const float* s = snap + (size_t)r.ia * ADJ_SNAP;
		A.dp = gv( s[4], s[5] );
		A.dq = grot( s[6], s[7] );
	}
	if ( snap && r.ib >= 0 )
	{
		const float* s = snap + (size_t)r.ib * ADJ_SNAP;
		B.dp = gv( s[4], s[5] );
		B.dq = grot( s[6], s[7] );
	}
	float* gA = r.ia >= 0 ? L.bodyAdj + (size_t)r.ia * ADJ_BODY : nullptr;
	float* gB = r.ib >= 0 ? L.bodyAdj + (size_t)r.ib * ADJ_BODY : nullptr;
	BodyV aA = { gA ? gA[4] : 0.0f, gA ? gA[5] : 0.0f, gA ? gA[6] : 0.0f };
	BodyV aB = { gB ? gB[4] : 0.0f, gB ? gB[5] : 0.0f, gB ? gB[6] : 0.0f };
	RowAdj* ra = (RowAdj*)( L.radj + (size_t)k * ADJ_RADJ );
	RowAdj g = *ra;
	float dpA[2] = { 0.0f, 0.0f }, dqA[2] = { 0.0f, 0.0f }, dpB[2] = { 0.0f, 0.0f }, dqB[2] = { 0.0f, 0.0f };
	if ( phase == 0 )
		warm_vjp( r, aA, aB, g );
	else if ( phase == 3 )
		restitution_vjp( r, A, B, sc, aA, aB, g );
	else
		solve_vjp( r, A, B, phase == 1, sc, aA, aB, g, dpA, dqA, dpB, dqB, scalar );
	*ra = g;
	if ( gA )
	{
		gA[4] = aA.vx;
		gA[5] = aA.vy;
		gA[6] = aA.w;
		gA[7] += dpA[0];
		gA[8] += dpA[1];
		gA[9] += dqA[0];
		gA[10] += dqA[1];
	}
	if ( gB )
	{
		gB[4] = aB.vx;
		gB[5] = aB.vy;
		gB[6] = aB.w;
		gB[7] += dpB[0];
		gB[8] += dpB[1];
		gB[9] += dqB[0];
		gB[10] += dqB[1];
	}
}

/* Reverse of one stage: colours in reverse order, then the overflow rows in reverse
 * order.  snap: body snapshot holding the position deltas the stage used (solve and
 * relax). */
__device__ void reverse_stage( const AdjLayout& L, const b2gTapeStep& h, int R, int phase, int tapeIndex, const float* snap,
							   const b2gStepConst& sc )
{
	const float* tape = L.phase + (size_t)tapeIndex * R * ADJ_PHASE;
	for ( int a = h.activeCount - 1; a >= 0; --a )
	{
		int c = h.active[a];
		for ( int k = h.colorStart[c] + (int)threadIdx.x; k < h.colorStart[c + 1]; k += ADJ_WARP )
			reverse_row( L, tape, k, phase, snap, sc, false );
		__syncwarp();
	}
	if ( threadIdx.x == 0 )
	{
		for ( int k = h.colorStart[B2G_COLORS] - 1; k >= h.colorStart[B2G_OVERFLOW]; --k )
			reverse_row( L, tape, k, phase, snap, sc, true );
	}
	__syncwarp();
}

__device__ void snapshot( const AdjLayout& L, int N, int index )
{
	float* dst = L.snap + (size_t)index * N * ADJ_SNAP;
	for ( int b = threadIdx.x; b < N; b += ADJ_WARP )
		for ( int i = 0; i < ADJ_SNAP; ++i )
			dst[(size_t)b * ADJ_SNAP + i] = L.state[(size_t)b * ADJ_STATE + i];
	__syncwarp();
}

__global__ void __launch_bounds__( ADJ_WARP ) k_adjoint( const b2gAdjointItem* items )
{
	const b2gAdjointItem& it = items[blockIdx.x];
	const b2gDevWorld& W = it.W;
	const int lane = threadIdx.x;
	const int N = it.bodies;
	AdjLayout L;
	adj_layout( &L, it.scratch, N, it.maxRows < 1 ? 1 : it.maxRows, it.contactCap < 1 ? 1 : it.contactCap, ADJ_MAX_SUBSTEPS );
	int unsupported = 0, mismatches = 0, replayDiffs = 0;

	for ( int s = lane; s < it.shapes; s += ADJ_WARP )
		it.gradFriction[s] = 0.0f;
	for ( int c = lane; c < it.contactCap; c += ADJ_WARP )
	{
		L.lamStamp[c] = -1;
		L.prevStamp[c] = -1;
	}
	for ( int b = lane; b < N; b += ADJ_WARP )
		for ( int i = 0; i < ADJ_BODY; ++i )
			L.bodyAdj[(size_t)b * ADJ_BODY + i] = 0.0f;
	__syncwarp();

	for ( int ts = it.stepCount - 1; ts >= 0; --ts )
	{
		const b2gTapeStep h = it.steps[ts];
		const b2gStepConst sc = h.sc;
		const int R = h.rows;
		const int S = sc.subSteps;
		if ( h.solve == 0 || S > ADJ_MAX_SUBSTEPS )
		{
			unsupported += h.solve != 0 ? 1 : 0;
			continue;
		}
		if ( h.jointStart[B2G_COLORS] > 0 )
			unsupported += 1;
		const float* recB = it.tapeBodies + 4 * h.bodyOff;
		const b2gTapeRow* recR = it.tapeRows + h.rowOff;

		/* rows of the previous step, by contact id (for the warm-start impulse adjoint) */
		if ( ts > 0 )
		{
			const b2gTapeStep& hp = it.steps[ts - 1];
			for ( int k = lane; k < hp.rows; k += ADJ_WARP )
			{
				int cid = it.tapeRows[hp.rowOff + k].cid;
				L.prevRow[cid] = k;
				L.prevStamp[cid] = ts - 1;
			}
		}

		/* step start: bodies */
		for ( int b = lane; b < N; b += ADJ_WARP )
		{
			const float* o = recB + 16 * b;
			float* st = L.start + (size_t)b * ADJ_START;
			st[0] = o[8];
			st[1] = o[9];
			st[2] = o[6];
			st[3] = o[7];
			st[4] = o[10];
			st[5] = o[11];
			st[6] = o[4];
			st[7] = o[5];
			st[8] = o[12];
			float* x = L.state + (size_t)b * ADJ_STATE;
			x[0] = o[0];
			x[1] = o[1];
			x[2] = o[2];
			x[3] = o[3];
			x[4] = 0.0f;
			x[5] = 0.0f;
			x[6] = 1.0f;
			x[7] = 0.0f;
			if ( o[12] != 0.0f )
			{
				float4 ms = ( (const float4*)W.mass )[b];
				float4 fo = ( (const float4*)W.force )[b];
				fo = make_float4( o[13], o[14], o[15], fo.w );
				float4 ex = ( (const float4*)W.extent )[b];
				VelocityTerms v = velocity_terms( ms, fo, ex, sc );
				float* tm = L.terms + (size_t)b * ADJ_TERMS;
				tm[0] = v.lvd.x;
				tm[1] = v.lvd.y;
				tm[2] = v.avd;
				tm[3] = v.ld;
				tm[4] = v.ad;
			}
		}
		__syncwarp();

		/* rows: manifold Jacobian and preparation */
		const float4* mass = (const float4*)W.mass;
		for ( int k = lane; k < R; k += ADJ_WARP )
		{
			const b2gTapeRow& tr = recR[k];
			const b2gShapeGeo& gA = W.geo[tr.shapeA];
			const b2gShapeGeo& gB = W.geo[tr.shapeB];
			if ( gA.type == 4 )
				unsupported += 1; /* chain links have no manifold Jacobian here */
			else if ( manifold_jacobian( gA, gB, L.start + (size_t)gA.bodyId * ADJ_START, L.start + (size_t)gB.bodyId * ADJ_START, tr.ia >= 0,
										 tr.ib >= 0, tr.m, L.jac + (size_t)k * ADJ_JAC ) == false )
				mismatches += 1;
			float4 zero = make_float4( 0.0f, 0.0f, 0.0f, 0.0f );
			Row r;
			prepare_row( r, &tr.m, tr.ia, tr.ib, tr.ia >= 0 ? mass[tr.ia] : zero, tr.ib >= 0 ? mass[tr.ib] : zero, replay_state( L, tr.ia ),
						 replay_state( L, tr.ib ), tr.friction, tr.restitution, ( tr.ia < 0 || tr.ib < 0 ) ? sc.staticSoft : sc.contactSoft,
						 sc.enableWarmStarting ? 1.0f : 0.0f );
			store_row_rec( L, k, r );
			float* ra = L.radj + (size_t)k * ADJ_RADJ;
			for ( int i = 0; i < ADJ_RADJ; ++i )
				ra[i] = 0.0f;
		}
		__syncwarp();

		/* forward replay */
		for ( int sub = 0; sub < S; ++sub )
		{
			snapshot( L, N, 2 * sub );
			for ( int b = lane; b < N; b += ADJ_WARP )
			{
				if ( L.start[(size_t)b * ADJ_START + 8] == 0.0f )
					continue;
				DevState x = replay_state( L, b );
				const float* tm = L.terms + (size_t)b * ADJ_TERMS;
				VelocityTerms v;
				v.lvd = gv( tm[0], tm[1] );
				v.avd = tm[2];
				v.ld = tm[3];
				v.ad = tm[4];
				integrate_velocity( x, v, sc );
				replay_store_velocity( L, b, x );
			}
			__syncwarp();
			if ( sc.enableWarmStarting )
				replay_stage( L, h, R, 0, 3 * sub + 0, sc );
			replay_stage( L, h, R, 1, 3 * sub + 1, sc );
			snapshot( L, N, 2 * sub + 1 );
			for ( int b = lane; b < N; b += ADJ_WARP )
			{
				if ( L.start[(size_t)b * ADJ_START + 8] == 0.0f )
					continue;
				DevState x = replay_state( L, b );
				integrate_position( x, sc.h );
				float* st = L.state + (size_t)b * ADJ_STATE;
				st[4] = x.dp.x;
				st[5] = x.dp.y;
				st[6] = x.dq.c;
				st[7] = x.dq.s;
			}
			__syncwarp();
			replay_stage( L, h, R, 2, 3 * sub + 2, sc );
		}
		snapshot( L, N, 2 * S );
		replay_stage( L, h, R, 3, 3 * S, sc );

		/* the replayed step must end where the next recorded step starts */
		if ( ts + 1 < it.stepCount )
		{
			const float* next = it.tapeBodies + 4 * it.steps[ts + 1].bodyOff;
			for ( int b = lane; b < N; b += ADJ_WARP )
			{
				const float* st = L.start + (size_t)b * ADJ_START;
				if ( st[8] == 0.0f )
					continue;
				const float* x = L.state + (size_t)b * ADJ_STATE;
				const float* o = next + 16 * b;
				b2gRot qf = gnormrot( gmulrot( grot( x[6], x[7] ), grot( st[2], st[3] ) ) );
				bool ok = x[0] == o[0] && x[1] == o[1] && x[2] == o[2] && st[0] + x[4] == o[8] && st[1] + x[5] == o[9] && qf.c == o[6] &&
						  qf.s == o[7];
				replayDiffs += ok ? 0 : 1;
			}
		}

		/* seed: the loss gradient with respect to the state after the last step */
		if ( ts == it.stepCount - 1 )
		{
			for ( int b = lane; b < N; b += ADJ_WARP )
			{
				const float* st = L.start + (size_t)b * ADJ_START;
				if ( st[8] == 0.0f )
					continue;
				const float* fin = L.snap + ( (size_t)2 * S * N + b ) * ADJ_SNAP;
				/* final rotation q' = normalize( dq q ) */
				float qc = st[2], qs = st[3], dqc = fin[6], dqs = fin[7];
				b2gRot qf = gnormrot( gmulrot( grot( dqc, dqs ), grot( qc, qs ) ) );
				const float* gf = it.gradFinal + 6 * b;
				float* g = L.bodyAdj + (size_t)b * ADJ_BODY;
				float lcx = st[4], lcy = st[5];
				/* p = c - rotate( q, lc ); angle: dq/dangle = ( -q.s, q.c ) */
				g[0] = gf[0];
				g[1] = gf[1];
				g[2] = gf[2] * -qf.s - ( gf[0] * lcx + gf[1] * lcy );
				g[3] = gf[2] * qf.c - ( -gf[0] * lcy + gf[1] * lcx );
				g[4] = gf[3];
				g[5] = gf[4];
				g[6] = gf[5];
			}
			__syncwarp();
		}

		/* reverse: finalisation */
		for ( int b = lane; b < N; b += ADJ_WARP )
		{
			const float* st = L.start + (size_t)b * ADJ_START;
			float* g = L.bodyAdj + (size_t)b * ADJ_BODY;
			if ( st[8] == 0.0f )
			{
				for ( int i = 0; i < ADJ_BODY; ++i )
					g[i] = 0.0f;
				continue;
			}
			const float* fin = L.snap + ( (size_t)2 * S * N + b ) * ADJ_SNAP;
			finalize_vjp( st[2], st[3], fin[6], fin[7], g );
		}
		__syncwarp();

		/* reverse: stored impulses receive the next step's warm-start adjoint */
		for ( int k = lane; k < R; k += ADJ_WARP )
		{
			int cid = recR[k].cid;
			if ( L.lamStamp[cid] != ts )
				continue;
			RowAdj* ra = (RowAdj*)( L.radj + (size_t)k * ADJ_RADJ );
			const float* lam = L.lam + 4 * (size_t)cid;
			ra->ni[0] += lam[0];
			ra->ni[1] += lam[1];
			ra->ti[0] += lam[2];
			ra->ti[1] += lam[3];
		}
		__syncwarp();

		/* reverse: restitution, then the substeps */
		reverse_stage( L, h, R, 3, 3 * S, nullptr, sc );
		for ( int sub = S - 1; sub >= 0; --sub )
		{
			reverse_stage( L, h, R, 2, 3 * sub + 2, L.snap + (size_t)( 2 * sub + 2 ) * N * ADJ_SNAP, sc );
			for ( int b = lane; b < N; b += ADJ_WARP )
			{
				if ( L.start[(size_t)b * ADJ_START + 8] == 0.0f )
					continue;
				ip_vjp( L.snap + ( (size_t)( 2 * sub + 1 ) * N + b ) * ADJ_SNAP, sc.h, L.bodyAdj + (size_t)b * ADJ_BODY );
			}
			__syncwarp();
			reverse_stage( L, h, R, 1, 3 * sub + 1, L.snap + (size_t)( 2 * sub ) * N * ADJ_SNAP, sc );
			if ( sc.enableWarmStarting )
				reverse_stage( L, h, R, 0, 3 * sub + 0, nullptr, sc );
			for ( int b = lane; b < N; b += ADJ_WARP )
			{
				if ( L.start[(size_t)b * ADJ_START + 8] == 0.0f )
					continue;
				const float* tm = L.terms + (size_t)b * ADJ_TERMS;
				iv_vjp( L.snap + ( (size_t)( 2 * sub ) * N + b ) * ADJ_SNAP, make_float4( tm[0], tm[1], tm[2], tm[3] ), tm[4], sc,
						L.bodyAdj + (size_t)b * ADJ_BODY );
			}
			__syncwarp();
		}

		/* reverse: preparation and the manifold Jacobian, colour by colour so that no
		 * two lanes update one body, then the overflow rows one after another on lane 0 */
		for ( int a = 0; a <= h.activeCount; ++a )
		{
			const bool ov = a == h.activeCount;
			const int c = ov ? B2G_OVERFLOW : h.active[a];
			const int first = ov ? ( lane == 0 ? h.colorStart[c] : h.colorStart[c + 1] ) : h.colorStart[c] + lane;
			const int stride = ov ? 1 : ADJ_WARP;
			for ( int k = first; k < h.colorStart[c + 1]; k += stride )
			{
				const b2gTapeRow& tr = recR[k];
				Row r = load_row_rec( L, k );
				const RowAdj* ra = (const RowAdj*)( L.radj + (size_t)k * ADJ_RADJ );
				const float* s0 = L.snap; /* snapshot 0: step-start velocities */
				DevState sA = identity_state(), sB = identity_state();
				if ( tr.ia >= 0 )
				{
					sA.v = gv( s0[(size_t)tr.ia * ADJ_SNAP + 0], s0[(size_t)tr.ia * ADJ_SNAP + 1] );
					sA.w = s0[(size_t)tr.ia * ADJ_SNAP + 2];
				}
				if ( tr.ib >= 0 )
				{
					sB.v = gv( s0[(size_t)tr.ib * ADJ_SNAP + 0], s0[(size_t)tr.ib * ADJ_SNAP + 1] );
					sB.w = s0[(size_t)tr.ib * ADJ_SNAP + 2];
				}
				float* gA = tr.ia >= 0 ? L.bodyAdj + (size_t)tr.ia * ADJ_BODY : nullptr;
				float* gB = tr.ib >= 0 ? L.bodyAdj + (size_t)tr.ib * ADJ_BODY : nullptr;
				BodyV aA = { gA ? gA[4] : 0.0f, gA ? gA[5] : 0.0f, gA ? gA[6] : 0.0f };
				BodyV aB = { gB ? gB[4] : 0.0f, gB ? gB[5] : 0.0f, gB ? gB[6] : 0.0f };
				float mAdj[12], lamIn[4];
				prepare_vjp( r, sA, sB, *ra, sc.enableWarmStarting ? 1.0f : 0.0f, mAdj, aA, aB, lamIn );
				/* manifold adjoint -> body centres and angles */
				const float* J = L.jac + (size_t)k * ADJ_JAC;
				float gpos[6] = { 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f };
				for ( int o = 0; o < 12; ++o )
					for ( int d = 0; d < 6; ++d )
						gpos[d] += mAdj[o] * J[o * 6 + d];
				if ( gA )
				{
					const float* st = L.start + (size_t)tr.ia * ADJ_START;
					gA[0] += gpos[0];
					gA[1] += gpos[1];
					gA[2] += gpos[2] * -st[3];
					gA[3] += gpos[2] * st[2];
					gA[4] = aA.vx;
					gA[5] = aA.vy;
					gA[6] = aA.w;
				}
				if ( gB )
				{
					const float* st = L.start + (size_t)tr.ib * ADJ_START;
					gB[0] += gpos[3];
					gB[1] += gpos[4];
					gB[2] += gpos[5] * -st[3];
					gB[3] += gpos[5] * st[2];
					gB[4] = aB.vx;
					gB[5] = aB.vy;
					gB[6] = aB.w;
				}
				/* warm-start impulses came from the previous step's stored impulses of
				 * the points with the same feature id (reference src/contact.c:555-568) */
				if ( ts > 0 && L.prevStamp[tr.cid] == ts - 1 )
				{
					const b2gTapeRow& old = it.tapeRows[it.steps[ts - 1].rowOff + L.prevRow[tr.cid]];
					float* lam = L.lam + 4 * (size_t)tr.cid;
					if ( L.lamStamp[tr.cid] != ts - 1 )
					{
						lam[0] = lam[1] = lam[2] = lam[3] = 0.0f;
						L.lamStamp[tr.cid] = ts - 1;
					}
					for ( int j = 0; j < tr.m.count; ++j )
					{
						for ( int jo = 0; jo < old.m.count; ++jo )
						{
							if ( old.m.pts[jo].id == tr.m.pts[j].id )
							{
								lam[jo] += lamIn[j];
								lam[2 + jo] += lamIn[2 + j];
								break;
							}
						}
					}
				}
			}
			__syncwarp();
		}

		/* friction: mu_row = sqrt( muA muB ) */
		if ( lane == 0 )
		{
			for ( int k = 0; k < R; ++k )
			{
				const b2gTapeRow& tr = recR[k];
				float gmu = ( (const RowAdj*)( L.radj + (size_t)k * ADJ_RADJ ) )->mu;
				if ( gmu == 0.0f )
					continue;
				float muA = it.shapeFriction[tr.shapeA], muB = it.shapeFriction[tr.shapeB];
				if ( muA > 0.0f )
					it.gradFriction[tr.shapeA] += gmu * 0.5f * tr.friction / muA;
				if ( muB > 0.0f )
					it.gradFriction[tr.shapeB] += gmu * 0.5f * tr.friction / muB;
			}
		}
		/* position deltas start each step at zero: their adjoints end here */
		for ( int b = lane; b < N; b += ADJ_WARP )
		{
			float* g = L.bodyAdj + (size_t)b * ADJ_BODY;
			g[7] = g[8] = g[9] = g[10] = 0.0f;
		}
		__syncwarp();
	}

	/* gradient with respect to the state at the start of the first recorded step:
	 * p = c - rotate( q, lc ), angle with dq/dangle = ( -q.s, q.c ) */
	for ( int b = lane; b < N; b += ADJ_WARP )
	{
		const float* st = L.start + (size_t)b * ADJ_START;
		const float* g = L.bodyAdj + (size_t)b * ADJ_BODY;
		float* out = it.gradInitial + 6 * b;
		float qc = st[2], qs = st[3], lcx = st[4], lcy = st[5];
		out[0] = g[0];
		out[1] = g[1];
		out[2] = g[2] * -qs + g[3] * qc + g[0] * ( -qs * lcx - qc * lcy ) + g[1] * ( qc * lcx - qs * lcy );
		out[3] = g[4];
		out[4] = g[5];
		out[5] = g[6];
	}
	for ( int off = 16; off > 0; off >>= 1 )
	{
		unsupported += __shfl_down_sync( 0xffffffffu, unsupported, off );
		mismatches += __shfl_down_sync( 0xffffffffu, mismatches, off );
		replayDiffs += __shfl_down_sync( 0xffffffffu, replayDiffs, off );
	}
	if ( lane == 0 )
	{
		it.status[0] = unsupported;
		it.status[1] = mismatches + replayDiffs;
		it.status[2] = mismatches;
		it.status[3] = replayDiffs;
	}
}

extern "C" int b2gd_adjoint_launch( const b2gAdjointItem* dItems, int count, void* stream )
{
	if ( count <= 0 )
		return 0;
	k_adjoint<<<count, ADJ_WARP, 0, (cudaStream_t)stream>>>( dItems );
	return (int)cudaGetLastError();
}
