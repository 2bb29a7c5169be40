// Batched evaluation of f = -tr(U^dagger W), its gate gradients and its Hessian on
// the GPU: the trace over basis columns b (reference src/matchgate_target.c:397-513),
// one column per thread block at a time, all columns of a call in one launch.
//
// Parity sectors.  Every matchgate preserves the parity of the basis index, so the
// column W e_b lives in the 2^(L-1) amplitudes of b's parity sector, and so do all
// forward and backward states that contribute to f, the gradient or the Hessian
// (amplitudes of the other sector only ever meet zeros).  A sector amplitude with
// full index a is stored at compact index c = a >> 1; the dropped least significant
// bit (qubit L-1) follows from the parity.  Qubit q < L-1 is compact bit L-2-q.
// Each gate then maps, for every compact "quartet", one corner pair (x, w) with its
// corner block and one center pair (y, z) with its center block.
//
// Tiles and passes.  A column's sector lives in a per-block global slot.  A pass
// loads tiles of 2^kt amplitudes spanning kt "local" compact bits into shared
// memory, applies every gate of the pass whose bits are local, and stores the tile
// back; when the sector has at most kt bits there is one tile and one pass.  The
// host schedules the passes: target circuits are greedily reordered (commuting gates
// only) to fuse many gates per pass; the fitted circuit W keeps its order, so the
// Hessian's "later gate" relation is the reference's.
#include "mgcu_common.cuh"

#include <algorithm>
#include <cmath>
#include <array>
#include <map>
#include <memory>
#include <vector>

namespace {

constexpr int MAXKT = 14;   // at most 2^14 amplitudes per shared-memory tile
constexpr int MAXNB = 31;   // compact bits (L <= 32)
constexpr int MAXPM = 128;  // distinct gate matrices per target pass (staged in shared memory)
constexpr int MAXPG = 128;  // gates per target pass (k_target_w stages their records in shared memory)

struct PassRec
{
	int gbeg, gend;        // this pass's gates: GateRec[gbeg, gend)
	int nnl;               // number of nonlocal compact bits (tiles = 2^nnl)
	int lbits[MAXKT];      // local bit j -> compact bit
	int nlbits[MAXNB];     // nonlocal bits, ascending
};

// type 0: both wires compact (la: wire i, lb: wire j); type 1: wire j is the
// dropped qubit (la: wire i); type 2: wire i is the dropped qubit (lb: wire j).
// lc: an auxiliary local bit used to pair a corner and a center pair.
struct GateRec { int g, type, la, lb, lc; };

struct Sched
{
	std::vector<PassRec> pass;
	std::vector<GateRec> gate;
	std::vector<int> pass_of;   // gate -> pass
};

int compact_bit(int L, int q) { return q == L - 1 ? -1 : L - 2 - q; }

// Build the pass schedule of a gate sequence.  reorder = false keeps the sequential
// order (passes are contiguous runs); reorder = true greedily pulls ready gates (all
// earlier gates on both wires scheduled) that add the fewest new local bits.  The
// lowest `low` compact bits are local in every pass, so that the tile's global reads
// and writes use whole 32-byte sectors.  masks (optional, reorder only): per gate the
// wires of its Jordan-Wigner string; the gate keeps its order relative to every gate
// acting on one of them (its local bits are still its two wires only).
void schedule(int L, int kt, const int* wires, int ng, bool reorder, Sched& s, int low = 3, const unsigned* masks = nullptr)
{
	const int nb = L - 1;
	const int c0 = std::min(low, kt);
	s.pass.clear(); s.gate.clear(); s.pass_of.assign(ng, -1);

	std::vector<int> order;
	std::vector<std::vector<int>> passes_gates;
	std::vector<unsigned> passes_sets;
	auto bits_of = [&](int g) {
		unsigned m = 0;
		const int a = compact_bit(L, wires[2 * g]), b = compact_bit(L, wires[2 * g + 1]);
		if (a >= 0) m |= 1u << a;
		if (b >= 0) m |= 1u << b;
		return m;
	};
	const unsigned base_set = (nb <= kt) ? ((nb >= 32) ? 0xffffffffu : ((1u << nb) - 1)) : ((1u << c0) - 1);

	if (!reorder)
	{
		unsigned cur = base_set;
		std::vector<int> pg;
		for (int g = 0; g < ng; g++)
		{
			const unsigned nm = cur | bits_of(g);
			if (__builtin_popcount(nm) > kt && !pg.empty())
			{
				passes_gates.push_back(pg); passes_sets.push_back(cur);
				pg.clear(); cur = base_set | bits_of(g);
			}
			else cur = nm;
			pg.push_back(g);
		}
		passes_gates.push_back(pg); passes_sets.push_back(cur);
	}
	else
	{
		std::vector<std::vector<int>> onq(L);
		auto wset = [&](int g) {
			unsigned m = (1u << wires[2 * g]) | (1u << wires[2 * g + 1]);
			if (masks) m |= masks[g];
			return m;
		};
		for (int g = 0; g < ng; g++)
			for (int q = 0; q < L; q++)
				if (wset(g) & (1u << q)) onq[q].push_back(g);
		std::vector<size_t> fr(L, 0);
		int done = 0;
		while (done < ng || passes_gates.empty())
		{
			unsigned cur = base_set;
			std::vector<int> pg;
			for (;;)
			{
				int best = -1, bestnew = 99;
				for (int q = 0; q < L; q++)
				{
					if (fr[q] >= onq[q].size()) continue;
					const int g = onq[q][fr[q]];
					const unsigned ws = wset(g);
					bool ready = true;
					for (int q2 = 0; q2 < L && ready; q2++)
						if ((ws & (1u << q2)) && (fr[q2] >= onq[q2].size() || onq[q2][fr[q2]] != g)) ready = false;
					if (!ready) continue;
					const unsigned m = bits_of(g);
					const int nw = __builtin_popcount(m & ~cur);
					if (__builtin_popcount(cur | m) > kt) continue;
					if (nw < bestnew || (nw == bestnew && g < best)) { best = g; bestnew = nw; }
				}
				if (best < 0) break;
				cur |= bits_of(best);
				for (int q2 = 0; q2 < L; q2++)
					if (wset(best) & (1u << q2)) fr[q2]++;
				pg.push_back(best);
				done++;
			}
			passes_gates.push_back(pg); passes_sets.push_back(cur);
			if (pg.empty()) break;   // only for ng == 0
		}
	}

	for (size_t p = 0; p < passes_gates.size(); p++)
	{
		unsigned set = passes_sets[p];
		// pad the local set to kt bits with the lowest unused compact bits
		for (int b = 0; b < nb && __builtin_popcount(set) < std::min(kt, nb); b++) set |= 1u << b;
		PassRec pr;
		memset(&pr, 0, sizeof(pr));
		int nl = 0, nn = 0;
		int lpos[32];
		for (int b = 0; b < nb; b++)
		{
			if (set & (1u << b)) { lpos[b] = nl; pr.lbits[nl++] = b; }
			else { lpos[b] = -1; pr.nlbits[nn++] = b; }
		}
		pr.nnl = nn;
		pr.gbeg = (int)s.gate.size();
		for (int g : passes_gates[p])
		{
			GateRec r;
			const int a = compact_bit(L, wires[2 * g]), b = compact_bit(L, wires[2 * g + 1]);
			r.g = g;
			r.type = (a >= 0 && b >= 0) ? 0 : (b < 0 ? 1 : 2);
			r.la = a >= 0 ? lpos[a] : -1;
			r.lb = b >= 0 ? lpos[b] : -1;
			const int used = r.type == 1 ? r.la : r.lb;
			r.lc = (used == 0) ? 1 : 0;
			s.gate.push_back(r);
			s.pass_of[g] = (int)p;
		}
		pr.gend = (int)s.gate.size();
		s.pass.push_back(pr);
	}
}

// ------------------------------------------------------------------------------------
// device side
// ------------------------------------------------------------------------------------

__device__ __forceinline__ unsigned ins0u(unsigned t, int p) { return ((t >> p) << (p + 1)) | (t & ((1u << p) - 1u)); }

// shared-memory accesses by 32-bit shared-window address (ld/st.shared, no generic
// addressing), for the state types of the precision policies
__device__ __forceinline__ unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }
template <class T> __device__ __forceinline__ T lds(unsigned a);
template <class T> __device__ __forceinline__ void sts(unsigned a, const T& v);
template <> __device__ __forceinline__ float4 lds<float4>(unsigned a)
{
	float4 v;
	asm volatile("ld.shared.v4.f32 {%0, %1, %2, %3}, [%4];" : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w) : "r"(a) : "memory");
	return v;
}
template <> __device__ __forceinline__ void sts<float4>(unsigned a, const float4& v)
{
	asm volatile("st.shared.v4.f32 [%0], {%1, %2, %3, %4};" :: "r"(a), "f"(v.x), "f"(v.y), "f"(v.z), "f"(v.w) : "memory");
}
template <> __device__ __forceinline__ double2 lds<double2>(unsigned a)
{
	double2 v;
	asm volatile("ld.shared.v2.f64 {%0, %1}, [%2];" : "=d"(v.x), "=d"(v.y) : "r"(a) : "memory");
	return v;
}
template <> __device__ __forceinline__ void sts<double2>(unsigned a, const double2& v)
{
	asm volatile("st.shared.v2.f64 [%0], {%1, %2};" :: "r"(a), "d"(v.x), "d"(v.y) : "memory");
}
template <> __device__ __forceinline__ float2 lds<float2>(unsigned a)
{
	float2 v;
	asm volatile("ld.shared.v2.f32 {%0, %1}, [%2];" : "=f"(v.x), "=f"(v.y) : "r"(a) : "memory");
	return v;
}
template <> __device__ __forceinline__ void sts<float2>(unsigned a, const float2& v)
{
	asm volatile("st.shared.v2.f32 [%0], {%1, %2};" :: "r"(a), "f"(v.x), "f"(v.y) : "memory");
}

// Target gate record, precomputed on the host for a tile size and a block size
// (all offsets in bytes of the swizzled tile):
//   m   = { MW, MY, MZ, SCX }: a quartet's w, y, z slots are its x slot XOR MW, MY, MZ;
//         x itself moves by SCX when the quartet's base has odd parity (gates on the
//         dropped qubit pair by parity; SCX = 0 otherwise)
//   h.x = lo | hi << 5 | dpar << 10 | kind word << 13  (lo < hi: the local bits a quartet
//         spans; dpar: parities of the quartet offsets d1, d2, d4)
//   h.y = the gate's slot among its pass's matrices, h.z = d1, h.w = d2, d4 = the
//         offset of quartet 4 (QPT 8)
//   sl  = Jordan-Wigner string of the gate: local bits | dropped-qubit flag << 16 |
//         string parities of d1, d2, d4 << 17;  snl = its nonlocal compact bits
// where dk is the swizzled slot offset of quartet t + k * blockDim from quartet t.  A
// gate with a string has its off-diagonal entries negated on amplitudes whose string
// bits have odd parity (a gate conjugated by the controlled-Z of a removed fermionic
// swap).
//   act = the range of rho (see k_target_w) whose quartets the gate changes:
//         rho_min + 4 | (rho_max + 4) << 4 | 0x100 (0: the gate changes nothing)
struct TGate { int4 m; int4 h; int d4, sl, snl, act; };

struct ProgDev
{
	const PassRec* pass;
	const GateRec* gate;
	int npass;
};

template <class P>
struct Args
{
	typedef typename P::T T;
	int L, nb, kt;
	long S;                    // 2^(L-1)
	ProgDev W, U;
	const T* wm;               // W gate matrices [ngates][8]: c0..c3, k0..k3
	const T* wmi;              // their block inverses (k_columns_adj)
	T* ck;                     // k_columns_adj: per block, each pass's output state [npass][S]
	const T* um;               // target gate matrices
	const int* ukind;          // target block kinds (null: every block general)
	const TGate* utg;          // target gate records (k_target)
	const int2* upm;           // per target pass: offset into upmats (entries), matrix count
	const T* upmats;           // per-pass distinct target matrices [8 entries each]
	unsigned pm_off;           // byte offset of the staged matrices in shared memory
	unsigned wperm_off;        // k_target_w: byte offset of the popcount-sorted free-bit table
	int ngates;
	const T* dense;            // -conj(U e_b) columns, or null (then U is run)
	long dense_b0;
	long b0, b1;               // column range of this launch
	T* su;                     // per-block slots [grid][S]
	T* sw;
	T* cache;                  // forward inputs per gate
	T* dcache;                 // backward inputs per gate (Hessian)
	int cache_per_column;      // 1: cache slot b - b0, 0: slot blockIdx.x
	int want_grad;
	double* part_f;            // [grid][2]
	double* part_g;            // [grid][ngates][16]
	// Hessian
	const int* place;
	const double* place_w;     // [nplace][ngates]
	const int* pass_of;
	const int* block;          // [ngates]
	int nplace, mdim;          // mdim = 8 * nblocks
	int hgroup;                // 1: a placement is its gate's whole block (every gate of the block adds its placeholder term)
	double* part_h;            // [grid][mdim][mdim][2]
	T* sh;                     // per-block slot for placeholder states
	T* ucols;                  // k_target: output columns [b - b0][S]
};

// shared-memory layout: tile, then the two deposit tables, then reduction scratch
struct Smem
{
	unsigned* dlo;
	unsigned* dhi;
	double* red;
	int h;
};

template <class T>
__device__ __forceinline__ Smem smem_layout(char* base, int kt, T*& tile)
{
	Smem s;
	tile = reinterpret_cast<T*>(base);
	s.dlo = reinterpret_cast<unsigned*>(base + sizeof(T) * (1u << kt));
	s.dhi = s.dlo + 128;
	s.red = reinterpret_cast<double*>(s.dhi + 128);
	s.h = kt / 2;
	return s;
}

// local -> compact index tables for one pass (caller synchronises)
__device__ __forceinline__ void setup_pass(const PassRec& pr, int kt, Smem& s)
{
	const int h = s.h;
	for (int i = threadIdx.x; i < 128; i += blockDim.x)
	{
		unsigned lo = 0, hi = 0;
		for (int j = 0; j < h; j++) if (i & (1 << j)) lo |= 1u << pr.lbits[j];
		for (int j = 0; j < kt - h; j++) if (i & (1 << j)) hi |= 1u << pr.lbits[h + j];
		s.dlo[i] = lo;
		s.dhi[i] = hi;
	}
}

__device__ __forceinline__ unsigned nl_base(const PassRec& pr, unsigned tau)
{
	unsigned b = 0;
	for (int j = 0; j < pr.nnl; j++) if (tau & (1u << j)) b |= 1u << pr.nlbits[j];
	return b;
}

__device__ __forceinline__ unsigned gidx(const Smem& s, unsigned base, unsigned e)
{
	return base | s.dlo[e & ((1u << s.h) - 1u)] | s.dhi[e >> s.h];
}

// quartet q of a gate -> tile positions of x, w (corner pair) and y, z (center pair)
__device__ __forceinline__ void quartet(const GateRec& r, unsigned q, int tpar, unsigned& ex, unsigned& ew, unsigned& ey, unsigned& ez)
{
	if (r.type == 0)
	{
		const int lo = min(r.la, r.lb), hi = max(r.la, r.lb);
		const unsigned base = ins0u(ins0u(q, lo), hi);
		const unsigned A = 1u << r.la, B = 1u << r.lb;
		ex = base; ew = base | A | B; ey = base | B; ez = base | A;
	}
	else
	{
		const int l = (r.type == 1) ? r.la : r.lb;
		const int lo = min(l, r.lc), hi = max(l, r.lc);
		const unsigned base = ins0u(ins0u(q, lo), hi);
		const unsigned A = 1u << l, C = 1u << r.lc;
		const int s = (__popc(base) + tpar) & 1;   // dropped bit of the base amplitude
		if (r.type == 1)
		{
			const unsigned a0 = base, a1 = base | A, b0 = base | C, b1 = base | C | A;
			ex = s ? b0 : a0; ew = s ? b1 : a1; ey = s ? a0 : b0; ez = s ? a1 : b1;
		}
		else
		{
			ex = s ? (base | C) : base;
			ew = s ? (base | C | A) : (base | A);
			ey = s ? (base | A) : (base | C | A);
			ez = s ? base : (base | C);
		}
	}
}

// L2 prefetch of [p, p + bytes) by the whole block, one 128-byte line per request
// (generic addresses inside one allocation)
__device__ __forceinline__ void l2_prefetch_block(const void* p, size_t bytes)
{
	const char* c = static_cast<const char*>(p);
	for (size_t o = (size_t)threadIdx.x * 128; o < bytes; o += (size_t)blockDim.x * 128)
		asm volatile("prefetch.L2 [%0];" :: "l"(c + o));
}

template <class P> struct Red;
template <> struct Red<PrecD>
{
	typedef double R;
	__device__ static void split(const PrecD::Acc& a, R& re, R& im) { re = a.re; im = a.im; }
	__device__ static void add(R& a, R b) { a += b; }
	__device__ static R shfl(R a, int m) { return __shfl_xor_sync(0xffffffffu, a, m); }
	__device__ static double to_d(R a) { return a; }
};
template <> struct Red<PrecF>
{
	typedef float2 R;
	__device__ static void split(const PrecF::Acc& a, R& re, R& im) { re = make_float2(a.rh, a.rl); im = make_float2(a.ih, a.il); }
	__device__ static void add(R& a, R b) { ff_add(a.x, a.y, b.x, b.y); }
	__device__ static R shfl(R a, int m) { return make_float2(__shfl_xor_sync(0xffffffffu, a.x, m), __shfl_xor_sync(0xffffffffu, a.y, m)); }
	__device__ static double to_d(R a) { return (double)a.x + (double)a.y; }
};
template <> struct Red<PrecX> : Red<PrecF> {};

// Reduce 8 complex accumulators over the block and add w * (sum) to dst[0..15]
// (re, im interleaved).  Warp level: a reduce-scatter over 16 reals (16 adds per
// lane instead of 80); block level: fixed-order FP64 sums over warps.  One barrier per
// call: successive calls (counted in nred, uniform over the block) alternate between
// the two halves of red, and the warp that sums the partials rotates, so the sums and
// the global read-modify-write of dst overlap the caller's next gate.  The barrier also
// orders the caller's tile writes before the next gate's reads.  red holds
// 2 * (blockDim.x / 32) * 16 doubles.
template <class P>
__device__ void block_reduce8(const typename P::Acc (&a)[8], double* red, double* dst, double w, int& nred)
{
	typedef Red<P> RD;
	typename RD::R v[16];
#pragma unroll
	for (int e = 0; e < 8; e++) RD::split(a[e], v[2 * e], v[2 * e + 1]);
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
	for (int t = 0; t < 8; t++)
	{
		const bool up = lane & 16;
		typename RD::R send = up ? v[t] : v[t + 8], keep = up ? v[t + 8] : v[t];
		RD::add(keep, RD::shfl(send, 16));
		v[t] = keep;
	}
#pragma unroll
	for (int t = 0; t < 4; t++)
	{
		const bool up = lane & 8;
		typename RD::R send = up ? v[t] : v[t + 4], keep = up ? v[t + 4] : v[t];
		RD::add(keep, RD::shfl(send, 8));
		v[t] = keep;
	}
#pragma unroll
	for (int t = 0; t < 2; t++)
	{
		const bool up = lane & 4;
		typename RD::R send = up ? v[t] : v[t + 2], keep = up ? v[t + 2] : v[t];
		RD::add(keep, RD::shfl(send, 4));
		v[t] = keep;
	}
	{
		const bool up = lane & 2;
		typename RD::R send = up ? v[0] : v[1], keep = up ? v[1] : v[0];
		RD::add(keep, RD::shfl(send, 2));
		v[0] = keep;
	}
	RD::add(v[0], RD::shfl(v[0], 1));
	const int idx = ((lane >> 4) & 1) * 8 + ((lane >> 3) & 1) * 4 + ((lane >> 2) & 1) * 2 + ((lane >> 1) & 1);
	const int nw = blockDim.x >> 5;
	double* rh = red + (nred & 1) * nw * 16;
	if ((lane & 1) == 0) rh[warp * 16 + idx] = RD::to_d(v[0]);
	__syncthreads();
	if (warp == (nred >> 1) % nw && lane < 16)
	{
		double s = 0;
		for (int k = 0; k < nw; k++) s += rh[k * 16 + lane];
		dst[lane] += w * s;
	}
	nred++;
}

// reduction scratch of a block of `threads` threads (block_reduce8's two halves)
constexpr size_t red_bytes(int threads) { return (size_t)2 * (threads / 32) * 16 * sizeof(double); }

template <class P>
__device__ void block_reduce1(const typename P::Acc& a, double* red, double* dst)
{
	typedef Red<P> RD;
	typename RD::R re, im;
	RD::split(a, re, im);
	for (int m = 16; m > 0; m >>= 1) { RD::add(re, RD::shfl(re, m)); RD::add(im, RD::shfl(im, m)); }
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	if (lane == 0) { red[warp * 2] = RD::to_d(re); red[warp * 2 + 1] = RD::to_d(im); }
	__syncthreads();
	if (threadIdx.x < 2)
	{
		double s = 0;
		for (int k = 0; k < (int)(blockDim.x >> 5); k++) s += red[k * 2 + threadIdx.x];
		dst[threadIdx.x] += s;
	}
	__syncthreads();
}

template <class T>
struct Gate8 { T c0, c1, c2, c3, k0, k1, k2, k3; };

template <class T>
__device__ __forceinline__ Gate8<T> load_gate(const T* m, int g)
{
	Gate8<T> r;
	const T* p = m + (size_t)g * 8;
	r.c0 = p[0]; r.c1 = p[1]; r.c2 = p[2]; r.c3 = p[3];
	r.k0 = p[4]; r.k1 = p[5]; r.k2 = p[6]; r.k3 = p[7];
	return r;
}

// apply one gate to the tile (forward); optionally store each input amplitude to
// the gate's cache column first
template <class P>
__device__ __forceinline__ void gate_forward(typename P::T* tile, const GateRec& r, const Gate8<typename P::T>& G, int Q, int tpar,
	typename P::T* cache_g, const Smem& s, unsigned nlb, bool tile_order = false)
{
	for (unsigned q = threadIdx.x; q < (unsigned)Q; q += blockDim.x)
	{
		unsigned ex, ew, ey, ez;
		quartet(r, q, tpar, ex, ew, ey, ez);
		const typename P::T x = tile[ex], w = tile[ew], y = tile[ey], z = tile[ez];
		if (cache_g && tile_order)
		{
			// the cached state in tile order: the backward pass reads it back by local index
			cache_g[ex] = x; cache_g[ew] = w; cache_g[ey] = y; cache_g[ez] = z;
		}
		else if (cache_g)
		{
			cache_g[gidx(s, nlb, ex)] = x; cache_g[gidx(s, nlb, ew)] = w;
			cache_g[gidx(s, nlb, ey)] = y; cache_g[gidx(s, nlb, ez)] = z;
		}
		tile[ex] = P::madd2(G.k0, x, G.k1, w);
		tile[ew] = P::madd2(G.k2, x, G.k3, w);
		tile[ey] = P::madd2(G.c0, y, G.c1, z);
		tile[ez] = P::madd2(G.c2, y, G.c3, z);
	}
}

// Structured blocks of target gates, classified exactly on the host (see classify_block):
// identity blocks are skipped, swaps move data, diagonal blocks multiply once, and blocks
// whose entries are each real or imaginary take 2-term instead of 4-term dot products.
enum { BK_ID = 0, BK_SWAP = 1, BK_D1 = 2, BK_NEG1 = 3, BK_DIAG = 4, BK_ANTI = 5, BK_RI = 6, BK_GEN = 7 };

template <class P>
__device__ __forceinline__ void pair_kind(typename P::T* tile, unsigned p0, unsigned p1, int kind, unsigned rot,
	const typename P::T& m0, const typename P::T& m1, const typename P::T& m2, const typename P::T& m3)
{
	typedef typename P::T T;
	switch (kind)
	{
	case BK_ID: return;
	case BK_SWAP: { const T a = tile[p0], b = tile[p1]; tile[p0] = b; tile[p1] = a; return; }
	case BK_D1: tile[p1] = P::mul(m3, tile[p1]); return;
	case BK_NEG1: tile[p1] = P::neg(tile[p1]); return;
	case BK_DIAG: tile[p0] = P::mul(m0, tile[p0]); tile[p1] = P::mul(m3, tile[p1]); return;
	case BK_ANTI: { const T a = tile[p0], b = tile[p1]; tile[p0] = P::mul(m1, b); tile[p1] = P::mul(m2, a); return; }
	case BK_RI:
	{
		const T a = tile[p0], b = tile[p1];
		tile[p0] = P::madd2_ri(m0, rot & 1, a, m1, rot & 2, b);
		tile[p1] = P::madd2_ri(m2, rot & 4, a, m3, rot & 8, b);
		return;
	}
	default:
	{
		const T a = tile[p0], b = tile[p1];
		tile[p0] = P::madd2(m0, a, m1, b);
		tile[p1] = P::madd2(m2, a, m3, b);
	}
	}
}

// forward application of a target gate with classified blocks; kw = kind word
// (center kind | corner kind << 3 | center rot bits << 6 | corner rot bits << 10)
template <class P>
__device__ __forceinline__ void gate_forward_kinds(typename P::T* tile, const GateRec& r, const Gate8<typename P::T>& G, int kw, int Q, int tpar)
{
	const int kc = kw & 7, kk = (kw >> 3) & 7;
	const unsigned rc = (kw >> 6) & 15, rk = (kw >> 10) & 15;
	for (unsigned q = threadIdx.x; q < (unsigned)Q; q += blockDim.x)
	{
		unsigned ex, ew, ey, ez;
		quartet(r, q, tpar, ex, ew, ey, ez);
		pair_kind<P>(tile, ex, ew, kk, rk, G.k0, G.k1, G.k2, G.k3);
		pair_kind<P>(tile, ey, ez, kc, rc, G.c0, G.c1, G.c2, G.c3);
	}
}

// contraction of the derivative d (state after the gate, read from dsrc) with the
// state before the gate x: acc[e] += d_r x_s for the 8 block entries (a thread's
// quartets of one gate and tile, block-reduced right after)
template <class P>
__device__ __forceinline__ void contract_quartet(typename P::Acc (&acc)[8], typename P::T dx, typename P::T dw, typename P::T dy, typename P::T dz,
	typename P::T x, typename P::T w, typename P::T y, typename P::T z)
{
	P::acc_mul_add_short(acc[0], dy, y); P::acc_mul_add_short(acc[1], dy, z);
	P::acc_mul_add_short(acc[2], dz, y); P::acc_mul_add_short(acc[3], dz, z);
	P::acc_mul_add_short(acc[4], dx, x); P::acc_mul_add_short(acc[5], dx, w);
	P::acc_mul_add_short(acc[6], dw, x); P::acc_mul_add_short(acc[7], dw, w);
}

// ---- tile transfers ----
template <class P>
__device__ __forceinline__ void tile_load_basis(typename P::T* tile, int kt, const Smem& s, unsigned nlb, unsigned cb)
{
	for (unsigned e = threadIdx.x; e < (1u << kt); e += blockDim.x)
		tile[e] = (gidx(s, nlb, e) == cb) ? P::make(1.0, 0.0) : P::zero();
}

template <class P>
__device__ __forceinline__ void tile_load(typename P::T* tile, int kt, const Smem& s, unsigned nlb, const typename P::T* src)
{
	for (unsigned e = threadIdx.x; e < (1u << kt); e += blockDim.x) tile[e] = src[gidx(s, nlb, e)];
}

template <class P>
__device__ __forceinline__ void tile_store(const typename P::T* tile, int kt, const Smem& s, unsigned nlb, typename P::T* dst, bool negconj)
{
	for (unsigned e = threadIdx.x; e < (1u << kt); e += blockDim.x)
	{
		const typename P::T v = tile[e];
		dst[gidx(s, nlb, e)] = negconj ? P::negconj(v) : v;
	}
}

// run a forward program from e_cb into `slot` (the result, -conj'ed if requested,
// ends in slot)
template <class P>
__device__ void run_forward(const ProgDev& prog, const typename P::T* mats, int kt, int nb, int par, unsigned cb,
	typename P::T* tile, Smem& s, typename P::T* slot, bool negconj_end, const int* kinds = nullptr)
{
	const int Q = 1 << (kt - 2);
	for (int p = 0; p < prog.npass; p++)
	{
		const PassRec& pr = prog.pass[p];
		__syncthreads();
		setup_pass(pr, kt, s);
		__syncthreads();
		const unsigned ntile = 1u << pr.nnl;
		for (unsigned tau = 0; tau < ntile; tau++)
		{
			const unsigned nlb = nl_base(pr, tau);
			const int tpar = (__popc(nlb) + par) & 1;
			if (p == 0) tile_load_basis<P>(tile, kt, s, nlb, cb);
			else tile_load<P>(tile, kt, s, nlb, slot);
			__syncthreads();
			for (int gi = pr.gbeg; gi < pr.gend; gi++)
			{
				const GateRec r = prog.gate[gi];
				const Gate8<typename P::T> G = load_gate(mats, r.g);
				if (kinds) gate_forward_kinds<P>(tile, r, G, kinds[r.g], Q, tpar);
				else gate_forward<P>(tile, r, G, Q, tpar, nullptr, s, nlb);
				__syncthreads();
			}
			tile_store<P>(tile, kt, s, nlb, slot, negconj_end && p == prog.npass - 1);
			__syncthreads();
		}
	}
}

// ------------------------------------------------------------------------------------
// target sweep: -conj(U e_b) of a circuit target, one column per block at a time.
//
// The tile of this kernel is stored swizzled: local index e lives in slot tsw(e), whose
// low bits are XORed with two higher bits (16-byte amplitudes: bits 3, 4 -> masks 7, 3;
// 8-byte amplitudes: bits 4, 5 -> masks 15, 7).  The map is linear over XOR, so a
// quartet's four slots are one slot XOR three per-gate masks, and eight (sixteen)
// consecutive threads hit distinct 16-byte (8-byte) bank groups for every pair of gate
// bits except two.  Gate records are packed (TGate), prefetched one gate ahead, and
// each thread applies a gate to QPT quartets at once: loads first, then arithmetic,
// then stores, with the block-kind dispatch outside the quartet batch.
// ------------------------------------------------------------------------------------
template <int ES>
__host__ __device__ __forceinline__ unsigned tsw(unsigned e)
{
	return ES == 16 ? (e ^ (((e >> 3) & 1u) * 7u) ^ (((e >> 4) & 1u) * 3u))
	                : (e ^ (((e >> 4) & 1u) * 15u) ^ (((e >> 5) & 1u) * 7u));
}


// one 2x2 block on QPT pairs (slots x ^ m0, x ^ m1) of NC tiles td bytes apart (NC
// columns of equal parity sharing every index); SG: off-diagonal entries negated on the
// pairs with sg[k] == 1 (implemented by negating the off-diagonal inputs)
template <class P, int QPT, bool SG, int NC>
__device__ __forceinline__ void tgt_block(unsigned tb, unsigned td, const unsigned (&x)[QPT], unsigned m0, unsigned m1, int kind,
	unsigned rot, unsigned m, const unsigned (&sg)[QPT])
{
	typedef typename P::T T;
	T a[NC][QPT], b[NC][QPT];
#define TGT_AA(c, k) (tb + (c) * td + (x[k] ^ m0))
#define TGT_BA(c, k) (tb + (c) * td + (x[k] ^ m1))
#define TGT_LOAD_AB() _Pragma("unroll") for (int c = 0; c < NC; c++) _Pragma("unroll") for (int k = 0; k < QPT; k++) { a[c][k] = lds<T>(TGT_AA(c, k)); b[c][k] = lds<T>(TGT_BA(c, k)); }
#define TGT_LOAD_B() _Pragma("unroll") for (int c = 0; c < NC; c++) _Pragma("unroll") for (int k = 0; k < QPT; k++) b[c][k] = lds<T>(TGT_BA(c, k));
#define TGT_MAT(q) lds<T>(m + (q) * (unsigned)sizeof(T))
	switch (kind)
	{
	case BK_ID: return;
	case BK_SWAP:
		TGT_LOAD_AB()
#pragma unroll
		for (int c = 0; c < NC; c++)
#pragma unroll
			for (int k = 0; k < QPT; k++)
			{
				sts<T>(TGT_AA(c, k), SG ? P::negif(b[c][k], sg[k]) : b[c][k]);
				sts<T>(TGT_BA(c, k), SG ? P::negif(a[c][k], sg[k]) : a[c][k]);
			}
		return;
	case BK_NEG1:
		TGT_LOAD_B()
#pragma unroll
		for (int c = 0; c < NC; c++)
#pragma unroll
			for (int k = 0; k < QPT; k++) sts<T>(TGT_BA(c, k), P::neg(b[c][k]));
		return;
	case BK_D1:
	{
		const T c3 = TGT_MAT(3);
		TGT_LOAD_B()
#pragma unroll
		for (int c = 0; c < NC; c++)
#pragma unroll
			for (int k = 0; k < QPT; k++) sts<T>(TGT_BA(c, k), P::mul(c3, b[c][k]));
		return;
	}
	case BK_DIAG:
	{
		const T c0 = TGT_MAT(0), c3 = TGT_MAT(3);
		TGT_LOAD_AB()
#pragma unroll
		for (int c = 0; c < NC; c++)
#pragma unroll
			for (int k = 0; k < QPT; k++) { sts<T>(TGT_AA(c, k), P::mul(c0, a[c][k])); sts<T>(TGT_BA(c, k), P::mul(c3, b[c][k])); }
		return;
	}
	case BK_ANTI:
	{
		const T c1 = TGT_MAT(1), c2 = TGT_MAT(2);
		TGT_LOAD_AB()
#pragma unroll
		for (int c = 0; c < NC; c++)
#pragma unroll
			for (int k = 0; k < QPT; k++)
			{
				const T as = SG ? P::negif(a[c][k], sg[k]) : a[c][k], bs = SG ? P::negif(b[c][k], sg[k]) : b[c][k];
				sts<T>(TGT_AA(c, k), P::mul(c1, bs)); sts<T>(TGT_BA(c, k), P::mul(c2, as));
			}
		return;
	}
	case BK_RI:
	{
		const T c0 = TGT_MAT(0), c1 = TGT_MAT(1), c2 = TGT_MAT(2), c3 = TGT_MAT(3);
		TGT_LOAD_AB()
		if (rot == 6u)   // real diagonal, imaginary off-diagonal (hopping terms)
		{
#pragma unroll
			for (int c = 0; c < NC; c++)
#pragma unroll
				for (int k = 0; k < QPT; k++)
				{
					const T bs = SG ? P::negif(b[c][k], sg[k]) : b[c][k], as = SG ? P::negif(a[c][k], sg[k]) : a[c][k];
					sts<T>(TGT_AA(c, k), P::madd2_ri(c0, false, a[c][k], c1, true, bs));
					sts<T>(TGT_BA(c, k), P::madd2_ri(c2, true, as, c3, false, b[c][k]));
				}
		}
		else
		{
#pragma unroll
			for (int c = 0; c < NC; c++)
#pragma unroll
				for (int k = 0; k < QPT; k++)
				{
					const T bs = SG ? P::negif(b[c][k], sg[k]) : b[c][k], as = SG ? P::negif(a[c][k], sg[k]) : a[c][k];
					sts<T>(TGT_AA(c, k), P::madd2_ri(c0, rot & 1, a[c][k], c1, rot & 2, bs));
					sts<T>(TGT_BA(c, k), P::madd2_ri(c2, rot & 4, as, c3, rot & 8, b[c][k]));
				}
		}
		return;
	}
	default:
	{
		const T c0 = TGT_MAT(0), c1 = TGT_MAT(1), c2 = TGT_MAT(2), c3 = TGT_MAT(3);
		TGT_LOAD_AB()
#pragma unroll
		for (int c = 0; c < NC; c++)
#pragma unroll
			for (int k = 0; k < QPT; k++)
			{
				const T bs = SG ? P::negif(b[c][k], sg[k]) : b[c][k], as = SG ? P::negif(a[c][k], sg[k]) : a[c][k];
				sts<T>(TGT_AA(c, k), P::madd2(c0, a[c][k], c1, bs));
				sts<T>(TGT_BA(c, k), P::madd2(c2, as, c3, b[c][k]));
			}
	}
	}
#undef TGT_AA
#undef TGT_BA
#undef TGT_LOAD_AB
#undef TGT_LOAD_B
#undef TGT_MAT
}

// a symmetric hop block [[c, i s], [i s, c]] on QPT pairs (slots x ^ m0, x ^ m1) of NC
// tiles; SG: s negated on the pairs with sg[k] == 1 (a Jordan-Wigner string of odd parity)
template <class P, int QPT, bool SG, int NC>
__device__ __forceinline__ void tgt_hop(unsigned tb, unsigned td, const unsigned (&x)[QPT], unsigned m0, unsigned m1,
	unsigned m, const unsigned (&sg)[QPT])
{
	typedef typename P::T T;
	const T c0 = lds<T>(m), c1 = lds<T>(m + (unsigned)sizeof(T));
	T a[NC][QPT], b[NC][QPT];
#pragma unroll
	for (int c = 0; c < NC; c++)
#pragma unroll
		for (int k = 0; k < QPT; k++)
		{
			a[c][k] = lds<T>(tb + c * td + (x[k] ^ m0));
			b[c][k] = lds<T>(tb + c * td + (x[k] ^ m1));
		}
#pragma unroll
	for (int c = 0; c < NC; c++)
#pragma unroll
		for (int k = 0; k < QPT; k++)
		{
			P::hop(c0, c1, SG ? sg[k] : 0u, a[c][k], b[c][k]);
			sts<T>(tb + c * td + (x[k] ^ m0), a[c][k]);
			sts<T>(tb + c * td + (x[k] ^ m1), b[c][k]);
		}
}

// kind word of a gate (host classification): center kind | corner kind << 3 | center rot
// << 6 | corner rot << 10 | symmetric-hop flags (center << 14, corner << 15)
__device__ __forceinline__ bool kw_hop_center(int kw) { return (kw & 7) == 6 && ((kw >> 6) & 15) == 6 && ((kw >> 14) & 1); }

// one target gate on the tile: QPT quartets per thread, q = t + k * blockDim.x
// (QPT * blockDim.x == number of quartets); nlb: the tile's nonlocal compact bits
template <class P, int QPT, int NC>
__device__ __forceinline__ void tgt_gate(unsigned tb, unsigned td, const TGate& r, unsigned mats, int tpar, unsigned nlb)
{
	constexpr int ES = sizeof(typename P::T);
	const unsigned MW = r.m.x, MY = r.m.y, MZ = r.m.z, SCX = r.m.w;
	const int lo = r.h.x & 31, hi = (r.h.x >> 5) & 31;
	const unsigned dpar = (unsigned)(r.h.x >> 10) & 7u;
	const unsigned b0 = ins0u(ins0u(threadIdx.x, lo), hi);
	const unsigned sb0 = tsw<ES>(b0) * ES;
	const unsigned p0 = (unsigned)(__popc(b0) + tpar) & 1u;
	const unsigned d1 = r.h.z, d2 = r.h.w, d4 = r.d4;
	unsigned x[QPT];
	if (SCX == 0)
	{
		// gates on two compact wires: the quartets' x slots are plain offsets
#pragma unroll
		for (int k = 0; k < QPT; k++) x[k] = sb0 ^ ((k & 1) ? d1 : 0u) ^ ((k & 2) ? d2 : 0u) ^ ((k & 4) ? d4 : 0u);
	}
	else
	{
#pragma unroll
		for (int k = 0; k < QPT; k++)
		{
			const unsigned dk = ((k & 1) ? d1 : 0u) ^ ((k & 2) ? d2 : 0u) ^ ((k & 4) ? d4 : 0u);
			const unsigned pk = p0 ^ (((k & 1) ? dpar : 0u) & 1u) ^ (((k & 2) ? (dpar >> 1) : 0u) & 1u) ^ (((k & 4) ? (dpar >> 2) : 0u) & 1u);
			x[k] = sb0 ^ dk ^ (pk ? SCX : 0u);
		}
	}
	const int kw = r.h.x >> 13;
	const unsigned m = mats + (unsigned)r.h.y * 8u * (unsigned)ES;   // the gate's staged matrix
	unsigned sg[QPT];
	if (r.sl | r.snl)
	{
		// parity of the string bits of each quartet's corner pair; the string bits are
		// not among the quartet's two bits, except that a string through the dropped
		// qubit (gates on two compact wires only) differs by one between the corner and
		// the center pair
		const unsigned ml = (unsigned)r.sl & 0xffffu, md = ((unsigned)r.sl >> 16) & 1u, sp = ((unsigned)r.sl >> 17) & 7u;
		const unsigned s0 = (unsigned)(__popc(b0 & ml) + __popc(nlb & (unsigned)r.snl)) ^ (md ? p0 : 0u);
#pragma unroll
		for (int k = 0; k < QPT; k++)
			sg[k] = (s0 ^ ((k & 1) ? sp : 0u) ^ ((k & 2) ? (sp >> 1) : 0u) ^ ((k & 4) ? (sp >> 2) : 0u)) & 1u;
		tgt_block<P, QPT, true, NC>(tb, td, x, 0u, MW, (kw >> 3) & 7, (kw >> 10) & 15, m + 4 * ES, sg);
#pragma unroll
		for (int k = 0; k < QPT; k++) sg[k] ^= md;
		if (kw_hop_center(kw)) tgt_hop<P, QPT, true, NC>(tb, td, x, MY, MZ, m, sg);
		else tgt_block<P, QPT, true, NC>(tb, td, x, MY, MZ, kw & 7, (kw >> 6) & 15, m, sg);
	}
	else
	{
		tgt_block<P, QPT, false, NC>(tb, td, x, 0u, MW, (kw >> 3) & 7, (kw >> 10) & 15, m + 4 * ES, sg);
		if (kw_hop_center(kw)) tgt_hop<P, QPT, false, NC>(tb, td, x, MY, MZ, m, sg);
		else tgt_block<P, QPT, false, NC>(tb, td, x, MY, MZ, kw & 7, (kw >> 6) & 15, m, sg);
	}
}

// the same with one quartet per iteration, for tiles whose quartet count is not 4 or 8
// times the block size
template <class P, int NC>
__device__ __forceinline__ void tgt_gate_any(unsigned tb, unsigned td, const TGate& r, unsigned mats, int tpar, unsigned nlb,
	unsigned Q)
{
	constexpr int ES = sizeof(typename P::T);
	const unsigned MW = r.m.x, MY = r.m.y, MZ = r.m.z, SCX = r.m.w;
	const int lo = r.h.x & 31, hi = (r.h.x >> 5) & 31;
	const int kw = r.h.x >> 13;
	const unsigned m = mats + (unsigned)r.h.y * 8u * (unsigned)ES;
	const unsigned ml = (unsigned)r.sl & 0xffffu, md = ((unsigned)r.sl >> 16) & 1u;
	const unsigned sn = (unsigned)__popc(nlb & (unsigned)r.snl);
	for (unsigned q = threadIdx.x; q < Q; q += blockDim.x)
	{
		const unsigned e = ins0u(ins0u(q, lo), hi);
		const unsigned pe = (unsigned)(__popc(e) + tpar) & 1u;
		const unsigned x[1] = { (tsw<ES>(e) * ES) ^ (pe ? SCX : 0u) };
		const unsigned sgk[1] = { ((unsigned)__popc(e & ml) + sn + (md ? pe : 0u)) & 1u };
		const unsigned sgc[1] = { sgk[0] ^ md };
		tgt_block<P, 1, true, NC>(tb, td, x, 0u, MW, (kw >> 3) & 7, (kw >> 10) & 15, m + 4 * ES, sgk);
		// the same arithmetic as the other sweep paths (hops by tgt_hop), so that every tile
		// and block size gives bit-identical columns
		if (kw_hop_center(kw)) tgt_hop<P, 1, true, NC>(tb, td, x, MY, MZ, m, sgc);
		else tgt_block<P, 1, true, NC>(tb, td, x, MY, MZ, kw & 7, (kw >> 6) & 15, m, sgc);
	}
}

// the gates [gbeg, gend) of a pass on one tile, records read one gate ahead
template <class P, int QPT, int NC>
__device__ __forceinline__ void tgt_gates(unsigned tb, unsigned td, const TGate* gates, int gbeg, int gend, unsigned mats,
	int tpar, unsigned nlb, unsigned Q)
{
	if (gbeg >= gend) return;
	TGate r = gates[gbeg];
	for (int gi = gbeg; gi < gend; gi++)
	{
		const TGate rn = gates[min(gi + 1, gend - 1)];
		if (QPT > 0) tgt_gate<P, (QPT > 0 ? QPT : 1), NC>(tb, td, r, mats, tpar, nlb);
		else tgt_gate_any<P, NC>(tb, td, r, mats, tpar, nlb, Q);
		__syncthreads();
		r = rn;
	}
}

// ------------------------------------------------------------------------------------
// Weight-restricted target sweep (k_target_w), for targets whose every gate conserves the
// Hamming weight (corner blocks diagonal: hopping and interaction terms of particle-
// conserving Hamiltonians, fermionic swaps).  U e_b then lives on the amplitudes of weight
// |b|: compact indices c (qubit L-1 dropped) with popc(c) in {|b| - 1, |b|}.  The members
// of a gate's quartet have popcounts r + (0, 1, 1, 2) in some order (r: popcount of the
// quartet's free bits, the tile's nonlocal bits adding popc(nlb)), so whether a quartet
// holds a nonzero amplitude that the gate changes depends only on
// rho = r - (|b| - popc(nlb)), in [-3, 0]; the host stores that range per gate (TGate.act).
// The quartets of a range of r are one run of the free-bit values sorted by popcount (a
// table in shared memory), so each gate's live quartets are enumerated without divergence.
// The skipped quartets hold zeros the gate maps to zeros: results are bit-identical to
// the full sweep.
// ------------------------------------------------------------------------------------

// byte offset of the popcount starts after the sorted free-bit table (16-byte aligned)
__host__ __device__ constexpr unsigned wtab_start_off(int kt) { return ((2u << (kt - 2)) + 15u) & ~15u; }
// byte offset of the staged gate records of a pass (after 16 popcount starts)
__host__ __device__ constexpr unsigned wtab_rec_off(int kt) { return wtab_start_off(kt) + 16u * (unsigned)sizeof(int); }

// the free-bit values 0 .. 2^F - 1 sorted by popcount (ties by value) into perm, and
// start[r] = index of the first value of popcount r (start[F + 1] = 2^F); whole block
__device__ __forceinline__ void w_perm_setup(int F, unsigned short* perm, int* start)
{
	auto binom = [](int n, int k) {
		if (k < 0 || k > n) return 0;
		int c = 1;
		for (int i = 0; i < k; i++) c = c * (n - i) / (i + 1);
		return c;
	};
	const unsigned nq = 1u << F;
	for (unsigned v = threadIdx.x; v < nq; v += blockDim.x)
	{
		// rank among the values of the same popcount (combinatorial number system)
		int rank = 0, i = 0;
		for (int p = 0; p < F; p++)
			if (v & (1u << p)) rank += binom(p, ++i);
		int off = 0;
		for (int r = 0; r < i; r++) off += binom(F, r);
		perm[off + rank] = (unsigned short)v;
	}
	for (int r = threadIdx.x; r <= F + 1; r += blockDim.x)
	{
		int off = 0;
		for (int q = 0; q < r; q++) off += binom(F, q);
		start[r] = off;
	}
}

// NQ live quartets of a gate: the ones at popcount-sorted positions j + k * stride
template <class P, int NQ, bool SG>
__device__ __forceinline__ void tgt_quartets_w(unsigned tb, unsigned td, const TGate& r, unsigned m, int tpar, unsigned sn,
	const unsigned short* perm, unsigned j, unsigned stride)
{
	constexpr int ES = sizeof(typename P::T);
	const int lo = r.h.x & 31, hi = (r.h.x >> 5) & 31, kw = r.h.x >> 13;
	const unsigned SCX = r.m.w, ml = (unsigned)r.sl & 0xffffu, md = ((unsigned)r.sl >> 16) & 1u;
	unsigned x[NQ], sg[NQ];
#pragma unroll
	for (int k = 0; k < NQ; k++)
	{
		const unsigned e = ins0u(ins0u(perm[j + k * stride], lo), hi);
		const unsigned pe = (unsigned)(__popc(e) + tpar) & 1u;
		x[k] = (tsw<ES>(e) * ES) ^ (pe ? SCX : 0u);
		sg[k] = SG ? (((unsigned)__popc(e & ml) + sn + (md ? pe : 0u)) & 1u) : 0u;
	}
	tgt_block<P, NQ, SG, 1>(tb, td, x, 0u, (unsigned)r.m.x, (kw >> 3) & 7, (kw >> 10) & 15, m + 4 * ES, sg);
	if (SG)
#pragma unroll
		for (int k = 0; k < NQ; k++) sg[k] ^= md;
	if (kw_hop_center(kw)) tgt_hop<P, NQ, SG, 1>(tb, td, x, (unsigned)r.m.y, (unsigned)r.m.z, m, sg);
	else tgt_block<P, NQ, SG, 1>(tb, td, x, (unsigned)r.m.y, (unsigned)r.m.z, kw & 7, (kw >> 6) & 15, m, sg);
}

// one gate on the live quartets [j0, j1) of the popcount-sorted order, NQ (1 or 2) per
// iteration
template <class P, bool SG, int NQ>
__device__ __forceinline__ void tgt_gate_w(unsigned tb, unsigned td, const TGate& r, unsigned mats, int tpar, unsigned nlb,
	const unsigned short* perm, unsigned j0, unsigned j1)
{
	constexpr int ES = sizeof(typename P::T);
	const unsigned m = mats + (unsigned)r.h.y * 8u * (unsigned)ES;
	const unsigned sn = SG ? (unsigned)__popc(nlb & (unsigned)r.snl) : 0u;
	unsigned j = j0 + threadIdx.x;
	if (NQ == 2)
	{
		for (; j + blockDim.x < j1; j += 2 * blockDim.x) tgt_quartets_w<P, 2, SG>(tb, td, r, m, tpar, sn, perm, j, blockDim.x);
		if (j < j1) tgt_quartets_w<P, 1, SG>(tb, td, r, m, tpar, sn, perm, j, blockDim.x);
	}
	else
		for (; j < j1; j += blockDim.x) tgt_quartets_w<P, 1, SG>(tb, td, r, m, tpar, sn, perm, j, blockDim.x);
}

// the gates [gbeg, gend) of a pass on one tile of nonlocal bits nlb, for a column of weight
// wb; F free bits per quartet.  One barrier per gate that has live quartets in the tile.
template <class P, int NQ>
__device__ __forceinline__ void tgt_gates_w(unsigned tb, unsigned td, const TGate* gates, int gbeg, int gend, unsigned mats,
	int tpar, unsigned nlb, int wb, int F, const unsigned short* perm, const int* start)
{
	const int delta = wb - __popc(nlb);
	for (int gi = gbeg; gi < gend; gi++)
	{
		const TGate r = gates[gi];
		if (!(r.act & 0x100)) continue;
		const int rlo = max(0, delta + (r.act & 15) - 4), rhi = min(F, delta + ((r.act >> 4) & 15) - 4);
		if (rlo > rhi) continue;   // no live quartet in this tile (the same for the whole block)
		if (r.sl | r.snl) tgt_gate_w<P, true, NQ>(tb, td, r, mats, tpar, nlb, perm, (unsigned)start[rlo], (unsigned)start[rhi + 1]);
		else tgt_gate_w<P, false, NQ>(tb, td, r, mats, tpar, nlb, perm, (unsigned)start[rlo], (unsigned)start[rhi + 1]);
		__syncthreads();
	}
}

// -conj(U e_b) of NC basis columns bs (of equal parity) into outs (the whole block); QPT:
// quartets per thread and gate (0: any, one quartet per iteration).  Shared memory: NC
// tiles, then the deposit tables and scratch; the pass matrices at a.pm_off.
template <class P, int QPT, int NC, bool W = false>
__device__ __forceinline__ void tgt_column(const Args<P>& a, const long (&bs)[NC], typename P::T* const (&outs)[NC], char* smem_raw)
{
	typedef typename P::T T;
	constexpr int ES = sizeof(T);
	const int kt = a.kt;
	const unsigned n = 1u << kt, Q = n >> 2, td = n * ES;
	T* tile_last;
	Smem s = smem_layout<T>(smem_raw + (NC - 1) * td, kt, tile_last);
	const unsigned tb = smem_u32(smem_raw);                 // the tiles, by shared-window address
	T* pm = reinterpret_cast<T*>(smem_raw + a.pm_off);   // this pass's distinct matrices
	const unsigned pms = smem_u32(pm);
	const int par = __popcll(bs[0]) & 1;
	for (int p = 0; p < a.U.npass; p++)
	{
		const PassRec& pr = a.U.pass[p];
		__syncthreads();
		setup_pass(pr, kt, s);
		{
			const int2 mp = a.upm[p];
			for (int i = threadIdx.x; i < mp.y * 8; i += blockDim.x) pm[i] = a.upmats[mp.x + i];
		}
		if (W)
		{
			// this pass's gate records, read by every tile of the pass
			const int4* src = reinterpret_cast<const int4*>(a.utg + pr.gbeg);
			int4* dst = reinterpret_cast<int4*>(smem_raw + a.wperm_off + wtab_rec_off(kt));
			const int n4 = (pr.gend - pr.gbeg) * (int)(sizeof(TGate) / sizeof(int4));
			for (int i = threadIdx.x; i < n4; i += blockDim.x) dst[i] = src[i];
		}
		__syncthreads();
		const bool last = p == a.U.npass - 1;
		const unsigned ntile = 1u << pr.nnl;
		for (unsigned tau = 0; tau < ntile; tau++)
		{
			const unsigned nlb = nl_base(pr, tau);
			const int tpar = (__popc(nlb) + par) & 1;
#pragma unroll
			for (int c = 0; c < NC; c++)
			{
				const unsigned tile = tb + c * td;
				const T* out = outs[c];
				if (p == 0)
				{
					const unsigned cb = (unsigned)(bs[c] >> 1);
					for (unsigned e = threadIdx.x; e < n; e += blockDim.x)
						sts<T>(tile + tsw<ES>(e) * ES, (gidx(s, nlb, e) == cb) ? P::make(1.0, 0.0) : P::zero());
				}
				else
					for (unsigned e0 = threadIdx.x; e0 < n; e0 += 8 * blockDim.x)
					{
						T v[8];   // eight reads in flight
#pragma unroll
						for (int k = 0; k < 8; k++)
						{
							const unsigned e = e0 + k * blockDim.x;
							if (e < n) v[k] = out[gidx(s, nlb, e)];
						}
#pragma unroll
						for (int k = 0; k < 8; k++)
						{
							const unsigned e = e0 + k * blockDim.x;
							if (e < n) sts<T>(tile + tsw<ES>(e) * ES, v[k]);
						}
					}
			}
			__syncthreads();
			if (W)
				tgt_gates_w<P, QPT == 1 ? 1 : 2>(tb, td, reinterpret_cast<const TGate*>(smem_raw + a.wperm_off + wtab_rec_off(kt)), 0,
					pr.gend - pr.gbeg, pms, tpar, nlb, __popcll(bs[0]), kt - 2,
					reinterpret_cast<const unsigned short*>(smem_raw + a.wperm_off),
					reinterpret_cast<const int*>(smem_raw + a.wperm_off + wtab_start_off(kt)));
			else tgt_gates<P, QPT, NC>(tb, td, a.utg, pr.gbeg, pr.gend, pms, tpar, nlb, Q);
#pragma unroll
			for (int c = 0; c < NC; c++)
			{
				const unsigned tile = tb + c * td;
				T* out = outs[c];
				for (unsigned e = threadIdx.x; e < n; e += blockDim.x)
				{
					const T v = lds<T>(tile + tsw<ES>(e) * ES);
					out[gidx(s, nlb, e)] = last ? P::negconj(v) : v;
				}
			}
			__syncthreads();
		}
	}
}

template <class P, int QPT>
__device__ __forceinline__ void tgt_column(const Args<P>& a, long b, typename P::T* out, char* smem_raw)
{
	const long bs[1] = { b };
	typename P::T* const outs[1] = { out };
	tgt_column<P, QPT, 1>(a, bs, outs, smem_raw);
}

// one instantiation per (block size, quartets per thread), so that each keeps only its
// own path's registers: 256 threads with 4, 8 or any quartets; 512 with 2, 4 or any
template <class P, int NT, int QPT>
__global__ void __launch_bounds__(NT, (NT == 512 && QPT == 4) ? 1 : (NT == 128 ? 3 : 2)) k_target(Args<P> a)
{
	extern __shared__ __align__(16) char smem_raw[];
	for (long b = a.b0 + blockIdx.x; b < a.b1; b += gridDim.x)
		tgt_column<P, QPT>(a, b, a.ucols + (size_t)(b - a.b0) * a.S, smem_raw);
}

// the weight-restricted sweep (targets that conserve the Hamming weight): NT threads, NQ
// live quartets per thread and iteration, three blocks per SM: 128 x 2, or 256 x 1 (at most
// 85 registers; more warps per SM, half the quartets in flight per thread)
template <class P, int NT, int NQ>
__global__ void __launch_bounds__(NT, 3) k_target_w(Args<P> a)
{
	extern __shared__ __align__(16) char smem_raw[];
	w_perm_setup(a.kt - 2, reinterpret_cast<unsigned short*>(smem_raw + a.wperm_off),
		reinterpret_cast<int*>(smem_raw + a.wperm_off + wtab_start_off(a.kt)));
	for (long b = a.b0 + blockIdx.x; b < a.b1; b += gridDim.x)
	{
		const long bs[1] = { b };
		typename P::T* const outs[1] = { a.ucols + (size_t)(b - a.b0) * a.S };
		tgt_column<P, NQ, 1, true>(a, bs, outs, smem_raw);
	}
}

// bytes of k_target_w's tables after the staged matrices: the sorted free-bit values, the
// popcount starts and the records of one pass (at most maxg gates)
constexpr size_t wtab_bytes(int kt, int maxg) { return wtab_rec_off(kt) + (size_t)maxg * sizeof(TGate); }

template <class P>
static void (*w_kernel(int threads, int nq))(Args<P>)
{
	return (threads == 256 && nq == 1) ? k_target_w<P, 256, 1> : k_target_w<P, 128, 2>;
}

// two columns of equal parity per block (b, b ^ 3 within each aligned group of four),
// sharing every per-gate computation; columns outside whole groups one at a time
template <class P, int QPT>
__global__ void __launch_bounds__(256, 1) k_target2(Args<P> a)
{
	typedef typename P::T T;
	extern __shared__ __align__(16) char smem_raw[];
	const long g0 = (a.b0 + 3) >> 2, g1 = a.b1 >> 2;
	const long npair = g1 > g0 ? 2 * (g1 - g0) : 0;
	for (long j = blockIdx.x; j < npair; j += gridDim.x)
	{
		const long base = (g0 + (j >> 1)) << 2;
		const long bs[2] = { base + (j & 1), base + 3 - (j & 1) };
		T* const outs[2] = { a.ucols + (size_t)(bs[0] - a.b0) * a.S, a.ucols + (size_t)(bs[1] - a.b0) * a.S };
		tgt_column<P, QPT, 2>(a, bs, outs, smem_raw);
	}
	// the rest: [b0, 4 g0) and [4 g1, b1), or all of [b0, b1) without a whole group
	const long r0 = npair ? min(a.b1, g0 << 2) - a.b0 : a.b1 - a.b0;
	const long r1 = npair ? a.b1 - (g1 << 2) : 0;
	for (long j = (long)gridDim.x - 1 - blockIdx.x; j < r0 + r1; j += gridDim.x)
	{
		const long b = j < r0 ? a.b0 + j : (g1 << 2) + (j - r0);
		tgt_column<P, QPT>(a, b, a.ucols + (size_t)(b - a.b0) * a.S, smem_raw);
	}
}

// the k_target instantiation for a tile of 2^kt amplitudes, a block size and columns per
// block (2: k_target2, 256 threads)
template <class P>
static void (*target_kernel(int kt, int threads, int nc = 1))(Args<P>)
{
	const long q = (1L << (kt - 2)) / threads, exact = (1L << (kt - 2)) % threads == 0;
	if (nc == 2) return (exact && q == 4) ? k_target2<P, 4> : (exact && q == 8) ? k_target2<P, 8> : k_target2<P, 0>;
	if (threads > 256) return (exact && q == 2) ? k_target<P, 512, 2> : (exact && q == 4) ? k_target<P, 512, 4> : k_target<P, 512, 0>;
	if (threads == 128 && exact && q == 8) return k_target<P, 128, 8>;
	if (exact && q == 4) return k_target<P, 256, 4>;
	if (exact && q == 8) return k_target<P, 256, 8>;
	return k_target<P, 256, 0>;
}


// ------------------------------------------------------------------------------------
// batched launches: work items (instance, column range) of many instances, taken by
// persistent blocks from an atomic counter in the order given (largest first); each
// item writes its own partial rows, so results do not depend on which block ran it
// ------------------------------------------------------------------------------------
struct BatchItem
{
	int inst;      // instance
	int slot;      // the item's partial row in its instance's part_f / part_g
	long b0, b1;   // columns
};

__device__ __forceinline__ int next_item(int* counter, int* shared_slot)
{
	if (threadIdx.x == 0) *shared_slot = atomicAdd(counter, 1);
	__syncthreads();
	const int it = *shared_slot;
	__syncthreads();
	return it;
}


// ------------------------------------------------------------------------------------
// stage A: per column -- W forward with cache, overlap, W backward; the target column
// comes from `dense` (k_target's output, a dense or host target) or, with WithU, from
// a sweep of the target program inside this kernel
// ------------------------------------------------------------------------------------
// one basis column b: target column from dense (or, WithU and no dense, the target
// program run into su), forward W with gate-input cache, overlap into facc, backward
// with gradient rows added to part_g row prow.  su, sw: the block's column slots;
// cache / dcache: this column's gate caches (null: none)
template <class P, bool WithU>
__device__ __forceinline__ void w_column(const Args<P>& a, long b, const typename P::T* dense, long dense_b0, long prow,
	typename P::T* su, typename P::T* sw, typename P::T* cache, typename P::T* dcache, typename P::Acc& facc, char* smem_raw)
{
	typedef typename P::T T;
	T* tile;
	Smem s = smem_layout<T>(smem_raw, a.kt, tile);
	const int kt = a.kt, Q = 1 << (kt - 2);
	const long S = a.S;
	{
		const int par = __popcll(b) & 1;
		const unsigned cb = (unsigned)(b >> 1);
		const T* dsrc;
		if (!WithU || dense) dsrc = dense + (size_t)(b - dense_b0) * S;
		else
		{
			run_forward<P>(a.U, a.um, kt, a.nb, par, cb, tile, s, su, true, a.ukind);
			dsrc = su;
		}

		// W forward, caching each gate's input; overlap on the last pass.  The caches of a
		// gate (its input here, the derivative entering it in the backward sweep) are kept
		// in tile order: tile tau of the gate's pass at offset tau * 2^kt, read back by
		// local index in the backward sweep and by the Hessian items
		const bool tl = true;
		for (int p = 0; p < a.W.npass; p++)
		{
			const PassRec& pr = a.W.pass[p];
			__syncthreads();
			setup_pass(pr, kt, s);
			__syncthreads();
			const unsigned ntile = 1u << pr.nnl;
			const bool last = (p == a.W.npass - 1);
			for (unsigned tau = 0; tau < ntile; tau++)
			{
				const unsigned nlb = nl_base(pr, tau);
				const int tpar = (__popcll(nlb) + par) & 1;
				if (p == 0) tile_load_basis<P>(tile, kt, s, nlb, cb);
				else tile_load<P>(tile, kt, s, nlb, sw);
				__syncthreads();
				for (int gi = pr.gbeg; gi < pr.gend; gi++)
				{
					const GateRec r = a.W.gate[gi];
					const Gate8<T> G = load_gate(a.wm, r.g);
					gate_forward<P>(tile, r, G, Q, tpar, cache ? cache + (size_t)r.g * S + (tl ? ((size_t)tau << kt) : 0) : nullptr,
						s, nlb, tl);
					__syncthreads();
				}
				if (last)
				{
					for (unsigned e = threadIdx.x; e < (1u << kt); e += blockDim.x)
						P::acc_mul_add(facc, dsrc[gidx(s, nlb, e)], tile[e]);
				}
				else tile_store<P>(tile, kt, s, nlb, sw, false);
				__syncthreads();
			}
		}

		if (!a.want_grad) return;

		// W backward: tile holds the derivative after the gate
		int nred = 0;
		for (int p = a.W.npass - 1; p >= 0; p--)
		{
			const PassRec& pr = a.W.pass[p];
			__syncthreads();
			setup_pass(pr, kt, s);
			__syncthreads();
			const unsigned ntile = 1u << pr.nnl;
			for (unsigned tau = 0; tau < ntile; tau++)
			{
				const unsigned nlb = nl_base(pr, tau);
				const int tpar = (__popcll(nlb) + par) & 1;
				// the cached inputs of this tile's gates (tile order, 2^kt contiguous
				// amplitudes each) go to L2 one gate ahead of their reads
				if (tl && pr.gend > pr.gbeg)
					l2_prefetch_block(cache + (size_t)a.W.gate[pr.gend - 1].g * S + ((size_t)tau << kt), sizeof(T) << kt);
				tile_load<P>(tile, kt, s, nlb, (p == a.W.npass - 1) ? dsrc : su);
				__syncthreads();
				for (int gi = pr.gend - 1; gi >= pr.gbeg; gi--)
				{
					const GateRec r = a.W.gate[gi];
					if (tl && gi > pr.gbeg)
						l2_prefetch_block(cache + (size_t)a.W.gate[gi - 1].g * S + ((size_t)tau << kt), sizeof(T) << kt);
					const Gate8<T> G = load_gate(a.wm, r.g);
					const T* cg = cache + (size_t)r.g * S;
					T* dg = dcache ? dcache + (size_t)r.g * S : nullptr;
					typename P::Acc acc[8];
#pragma unroll
					for (int e = 0; e < 8; e++) acc[e] = P::acc_zero();
					if (tl && (unsigned)Q % blockDim.x == 0)
					{
						// cache in tile order, read one quartet ahead of the arithmetic
						const T* ct = cg + ((size_t)tau << kt);
						const unsigned nq = (unsigned)Q / blockDim.x;
						unsigned ex, ew, ey, ez;
						quartet(r, threadIdx.x, tpar, ex, ew, ey, ez);
						T cx = ct[ex], cw = ct[ew], cy = ct[ey], cz = ct[ez];
						for (unsigned k = 0; k < nq; k++)
						{
							const unsigned fx = ex, fw = ew, fy = ey, fz = ez;
							const T x0 = cx, w0 = cw, y0 = cy, z0 = cz;
							if (k + 1 < nq)
							{
								quartet(r, threadIdx.x + (k + 1) * blockDim.x, tpar, ex, ew, ey, ez);
								cx = ct[ex]; cw = ct[ew]; cy = ct[ey]; cz = ct[ez];
							}
							const T dx = tile[fx], dw = tile[fw], dy = tile[fy], dz = tile[fz];
							if (dg)
							{
								T* dt = dg + ((size_t)tau << kt);
								dt[fx] = dx; dt[fw] = dw; dt[fy] = dy; dt[fz] = dz;
							}
							contract_quartet<P>(acc, dx, dw, dy, dz, x0, w0, y0, z0);
							tile[fx] = P::madd2(G.k0, dx, G.k2, dw);
							tile[fw] = P::madd2(G.k1, dx, G.k3, dw);
							tile[fy] = P::madd2(G.c0, dy, G.c2, dz);
							tile[fz] = P::madd2(G.c1, dy, G.c3, dz);
						}
					}
					else
					for (unsigned q = threadIdx.x; q < (unsigned)Q; q += blockDim.x)
					{
						unsigned ex, ew, ey, ez;
						quartet(r, q, tpar, ex, ew, ey, ez);
						const unsigned gx = gidx(s, nlb, ex), gw = gidx(s, nlb, ew), gy = gidx(s, nlb, ey), gz = gidx(s, nlb, ez);
						const T dx = tile[ex], dw = tile[ew], dy = tile[ey], dz = tile[ez];
						if (dg)
						{
							T* dt = dg + ((size_t)tau << kt);
							dt[ex] = dx; dt[ew] = dw; dt[ey] = dy; dt[ez] = dz;
						}
						if (tl)
						{
							const T* ct = cg + ((size_t)tau << kt);
							contract_quartet<P>(acc, dx, dw, dy, dz, ct[ex], ct[ew], ct[ey], ct[ez]);
						}
						else contract_quartet<P>(acc, dx, dw, dy, dz, cg[gx], cg[gw], cg[gy], cg[gz]);
						// transpose (no conjugation): reference src/gate.c:725-728
						tile[ex] = P::madd2(G.k0, dx, G.k2, dw);
						tile[ew] = P::madd2(G.k1, dx, G.k3, dw);
						tile[ey] = P::madd2(G.c0, dy, G.c2, dz);
						tile[ez] = P::madd2(G.c1, dy, G.c3, dz);
					}
					block_reduce8<P>(acc, s.red, a.part_g + ((size_t)prow * a.ngates + r.g) * 16, 1.0, nred);
				}
				if (p > 0) tile_store<P>(tile, kt, s, nlb, su, false);
				__syncthreads();
			}
		}
	}
}

template <class P, bool WithU>
__global__ void __launch_bounds__(256, 2) k_columns(Args<P> a)
{
	typedef typename P::T T;
	extern __shared__ __align__(16) char smem_raw[];
	const long S = a.S;
	typename P::Acc facc = P::acc_zero();
	T* su = a.su + (size_t)blockIdx.x * S;
	T* sw = a.sw + (size_t)blockIdx.x * S;
	for (long b = a.b0 + blockIdx.x; b < a.b1; b += gridDim.x)
	{
		const long slot = a.cache_per_column ? (b - a.b0) : blockIdx.x;
		T* cache = a.cache ? a.cache + (size_t)slot * a.ngates * S : nullptr;
		T* dcache = a.dcache ? a.dcache + (size_t)slot * a.ngates * S : nullptr;
		w_column<P, WithU>(a, b, a.dense, a.dense_b0, blockIdx.x, su, sw, cache, dcache, facc, smem_raw);
	}
	T* tile;
	Smem s = smem_layout<T>(smem_raw, a.kt, tile);
	block_reduce1<P>(facc, s.red, a.part_f + (size_t)blockIdx.x * 2);
}

// f and gate gradients of one column without cached gate inputs (gradient plans with
// invertible fitted gates): the forward sweep keeps each pass's output state (a checkpoint;
// the state is written at the end of every pass anyway, to hand it to the next pass), and the
// backward sweep reloads the output of the pass it is in and recovers each gate's input by
// applying the gate's block inverses (computed on the host), in the same quartet loop as the
// transposed derivative and the gradient contraction, so no barrier separates them.  Two
// tiles per block (the state and the derivative).  Reference: the backward sweep of
// src/matchgate_brickwall.c:87-127, whose inputs come from the forward cache there.
template <class P>
__device__ __forceinline__ void w_column_adj(const Args<P>& a, long b, long prow, typename P::T* su, typename P::T* ck,
	typename P::Acc& facc, char* smem_raw)
{
	typedef typename P::T T;
	const int kt = a.kt, Q = 1 << (kt - 2);
	T* ft = reinterpret_cast<T*>(smem_raw);   // the state
	T* tile;                                  // the forward sweep's state, then the derivative
	Smem s = smem_layout<T>(smem_raw + sizeof(T) * ((size_t)1 << kt), kt, tile);
	const long S = a.S;
	const int par = __popcll(b) & 1;
	const unsigned cb = (unsigned)(b >> 1);
	const T* dsrc = a.dense + (size_t)(b - a.dense_b0) * S;
	const int np = a.W.npass;
	for (int p = 0; p < np; p++)
	{
		const PassRec& pr = a.W.pass[p];
		__syncthreads();
		setup_pass(pr, kt, s);
		__syncthreads();
		const unsigned ntile = 1u << pr.nnl;
		const bool last = p == np - 1;
		for (unsigned tau = 0; tau < ntile; tau++)
		{
			const unsigned nlb = nl_base(pr, tau);
			const int tpar = (__popcll(nlb) + par) & 1;
			if (p == 0) tile_load_basis<P>(tile, kt, s, nlb, cb);
			else tile_load<P>(tile, kt, s, nlb, ck + (size_t)(p - 1) * S);
			__syncthreads();
			for (int gi = pr.gbeg; gi < pr.gend; gi++)
			{
				const GateRec r = a.W.gate[gi];
				gate_forward<P>(tile, r, load_gate(a.wm, r.g), Q, tpar, nullptr, s, nlb);
				__syncthreads();
			}
			if (last)
				for (unsigned e = threadIdx.x; e < (1u << kt); e += blockDim.x)
					P::acc_mul_add(facc, dsrc[gidx(s, nlb, e)], tile[e]);
			tile_store<P>(tile, kt, s, nlb, ck + (size_t)p * S, false);
			__syncthreads();
		}
	}
	int nred = 0;
	for (int p = np - 1; p >= 0; p--)
	{
		const PassRec& pr = a.W.pass[p];
		__syncthreads();
		setup_pass(pr, kt, s);
		__syncthreads();
		const unsigned ntile = 1u << pr.nnl;
		for (unsigned tau = 0; tau < ntile; tau++)
		{
			const unsigned nlb = nl_base(pr, tau);
			const int tpar = (__popcll(nlb) + par) & 1;
			tile_load<P>(tile, kt, s, nlb, (p == np - 1) ? dsrc : su);
			tile_load<P>(ft, kt, s, nlb, ck + (size_t)p * S);
			__syncthreads();
			for (int gi = pr.gend - 1; gi >= pr.gbeg; gi--)
			{
				const GateRec r = a.W.gate[gi];
				const Gate8<T> G = load_gate(a.wm, r.g), Gi = load_gate(a.wmi, r.g);
				typename P::Acc acc[8];
#pragma unroll
				for (int e = 0; e < 8; e++) acc[e] = P::acc_zero();
				for (unsigned q = threadIdx.x; q < (unsigned)Q; q += blockDim.x)
				{
					unsigned ex, ew, ey, ez;
					quartet(r, q, tpar, ex, ew, ey, ez);
					const T fx = ft[ex], fw = ft[ew], fy = ft[ey], fz = ft[ez];
					// the gate's input: its inverse applied to its output
					const T x = P::madd2(Gi.k0, fx, Gi.k1, fw), w = P::madd2(Gi.k2, fx, Gi.k3, fw);
					const T y = P::madd2(Gi.c0, fy, Gi.c1, fz), z = P::madd2(Gi.c2, fy, Gi.c3, fz);
					ft[ex] = x; ft[ew] = w; ft[ey] = y; ft[ez] = z;
					const T dx = tile[ex], dw = tile[ew], dy = tile[ey], dz = tile[ez];
					contract_quartet<P>(acc, dx, dw, dy, dz, x, w, y, z);
					// transpose (no conjugation): reference src/gate.c:725-728
					tile[ex] = P::madd2(G.k0, dx, G.k2, dw);
					tile[ew] = P::madd2(G.k1, dx, G.k3, dw);
					tile[ey] = P::madd2(G.c0, dy, G.c2, dz);
					tile[ez] = P::madd2(G.c1, dy, G.c3, dz);
				}
				block_reduce8<P>(acc, s.red, a.part_g + ((size_t)prow * a.ngates + r.g) * 16, 1.0, nred);
			}
			if (p > 0) tile_store<P>(tile, kt, s, nlb, su, false);
			__syncthreads();
		}
	}
}

// 128 threads, three blocks per SM: the state, the derivative, both gates' blocks and the
// eight accumulators fit in 168 registers without spilling
constexpr int ADJ_THREADS = 128;

template <class P>
__global__ void __launch_bounds__(ADJ_THREADS, 3) k_columns_adj(Args<P> a)
{
	typedef typename P::T T;
	extern __shared__ __align__(16) char smem_raw[];
	const long S = a.S;
	typename P::Acc facc = P::acc_zero();
	T* su = a.su + (size_t)blockIdx.x * S;
	T* ck = a.ck + (size_t)blockIdx.x * a.W.npass * S;
	for (long b = a.b0 + blockIdx.x; b < a.b1; b += gridDim.x)
		w_column_adj<P>(a, b, blockIdx.x, su, ck, facc, smem_raw);
	T* tile;
	Smem s = smem_layout<T>(smem_raw + sizeof(T) * ((size_t)1 << a.kt), a.kt, tile);
	block_reduce1<P>(facc, s.red, a.part_f + (size_t)blockIdx.x * 2);
}

// batched items of one tile class (quartets per thread in the target sweep: QPT), target
// and fitted circuit per column: the target column goes into the
// block's slot sx, then the fitted circuit runs against it; slots and gate cache live in
// per-block scratch (3 slots of slot_stride, then cache_stride elements)
template <class P, int QPT>
__global__ void __launch_bounds__(256, 2) k_batch(const Args<P>* __restrict__ args_t, const Args<P>* __restrict__ args_c,
	const BatchItem* __restrict__ items, int nitems, int* counter, typename P::T* scratch, long slot_stride, long cache_stride)
{
	typedef typename P::T T;
	extern __shared__ __align__(16) char smem_raw[];
	__shared__ int it_s;
	T* sx = scratch + (size_t)blockIdx.x * (3 * slot_stride + cache_stride);
	T* su = sx + slot_stride;
	T* sw = su + slot_stride;
	T* cache = sw + slot_stride;
	for (;;)
	{
		const int it = next_item(counter, &it_s);
		if (it >= nitems) break;
		const BatchItem I = items[it];
		const Args<P>& at = args_t[I.inst];
		const Args<P>& a = args_c[I.inst];
		typename P::Acc facc = P::acc_zero();
		for (long b = I.b0; b < I.b1; b++)
		{
			tgt_column<P, QPT>(at, b, sx, smem_raw);
			w_column<P, false>(a, b, sx, b, I.slot, su, sw, a.want_grad ? cache : nullptr, nullptr, facc, smem_raw);
		}
		T* tile;
		Smem s = smem_layout<T>(smem_raw, a.kt, tile);
		block_reduce1<P>(facc, s.red, a.part_f + (size_t)I.slot * 2);
	}
}

// ------------------------------------------------------------------------------------
// stage B: Hessian items (column, placement, entry): the placeholder state of one
// gate entry pushed through all later gates, contracted at each with the cached
// derivative (reference src/matchgate_brickwall.c:177-231).  Consecutive gates of a
// pass with the same block and weight (a brickwall layer) share one block reduction:
// the thread accumulators carry over, up to HESS_MERGE quartets per thread.
//
// Grouped placements (hgroup, the plain Hessian of parameter blocks shared by several
// gates, as the reference's per-layer brickwall Hessian): an item is (column, block,
// entry) and carries the derivative of the state with respect to that entry of the
// block's matrix, forward mode: it starts as the placeholder state at the block's first
// gate, and at every later gate s of the block, B <- G_s B + placeholder_s(input of s).
// Contracting B with the cached derivative at a gate s gives the sum over the block's
// gates r < s of what the per-gate items (r, entry) contribute there, so one item does
// the work of all the block's placements: at L=16 with 5 layers, 120 instead of 780
// gate steps per column and entry.  The same pairs (r < s) land in the same Hessian
// blocks, so the symmetrisation that follows is unchanged.
// ------------------------------------------------------------------------------------
constexpr int HESS_MERGE = 64;

template <class P>
__global__ void __launch_bounds__(256, 2) k_hessian(Args<P> a, long nitems)
{
	typedef typename P::T T;
	extern __shared__ __align__(16) char smem_raw[];
	T* tile;
	Smem s = smem_layout<T>(smem_raw, a.kt, tile);
	const int kt = a.kt, Q = 1 << (kt - 2);
	const long S = a.S;
	T* sh = a.sh + (size_t)blockIdx.x * S;
	double* parth = a.part_h + (size_t)blockIdx.x * a.mdim * a.mdim * 2;
	int nred = 0;
	const int qpt = (Q + (int)blockDim.x - 1) / (int)blockDim.x;
	typename P::Acc acc[8];
#pragma unroll
	for (int e = 0; e < 8; e++) acc[e] = P::acc_zero();
	int merged = 0;

	for (long it = blockIdx.x; it < nitems; it += gridDim.x)
	{
		const int x = (int)(it & 7);
		const long rest = it >> 3;
		const int p = (int)(rest % a.nplace);
		const long bi = rest / a.nplace;
		const long b = a.b0 + bi;
		const int par = __popcll(b) & 1;
		const int k = a.place[p];
		const int pk = a.pass_of[k];
		const T* cache = a.cache + (size_t)bi * a.ngates * S;
		const T* dcache = a.dcache + (size_t)bi * a.ngates * S;
		const double* wrow = a.place_w + (size_t)p * a.ngates;
		double* hrow = parth + (size_t)(a.block[k] * 8 + x) * a.mdim * 2;
		const int grp = a.hgroup ? a.block[k] : -1;
		for (int pp = pk; pp < a.W.npass; pp++)
		{
			const PassRec& pr = a.W.pass[pp];
			__syncthreads();
			setup_pass(pr, kt, s);
			__syncthreads();
			const unsigned ntile = 1u << pr.nnl;
			for (unsigned tau = 0; tau < ntile; tau++)
			{
				const unsigned nlb = nl_base(pr, tau);
				const int tpar = (__popcll(nlb) + par) & 1;
				if (pp == pk)
				{
					// the placement gate's input, cached in tile order
					const T* ct = cache + (size_t)k * S + ((size_t)tau << kt);
					for (unsigned e = threadIdx.x; e < (1u << kt); e += blockDim.x) tile[e] = ct[e];
				}
				else tile_load<P>(tile, kt, s, nlb, sh);
				__syncthreads();
				for (int gi = pr.gbeg; gi < pr.gend; gi++)
				{
					const GateRec r = a.W.gate[gi];
					if (r.g < k) continue;
					if (r.g == k)
					{
						// placeholder: the derivative of the gate's output w.r.t. entry x
						for (unsigned q = threadIdx.x; q < (unsigned)Q; q += blockDim.x)
						{
							unsigned ex, ew, ey, ez;
							quartet(r, q, tpar, ex, ew, ey, ez);
							const T vx = tile[ex], vw = tile[ew], vy = tile[ey], vz = tile[ez];
							const T zero = P::zero();
							T ox = zero, ow = zero, oy = zero, oz = zero;
							switch (x)
							{
							case 0: oy = vy; break;   // center (0,0)
							case 1: oy = vz; break;   // center (0,1)
							case 2: oz = vy; break;   // center (1,0)
							case 3: oz = vz; break;   // center (1,1)
							case 4: ox = vx; break;   // corner (0,0)
							case 5: ox = vw; break;   // corner (0,1)
							case 6: ow = vx; break;   // corner (1,0)
							default: ow = vw; break;  // corner (1,1)
							}
							tile[ex] = ox; tile[ew] = ow; tile[ey] = oy; tile[ez] = oz;
						}
						__syncthreads();
						continue;
					}
					const Gate8<T> G = load_gate(a.wm, r.g);
					const T* dg = dcache + (size_t)r.g * S + ((size_t)tau << kt);   // tile order
					const bool apply = (r.g != a.ngates - 1);
					// grouped placement: this gate of the block adds its placeholder term
					// (entry x of its input, cached in tile order) after the gate
					const T* cg = (grp >= 0 && a.block[r.g] == grp) ? cache + (size_t)r.g * S + ((size_t)tau << kt) : nullptr;
					const int blk = a.block[r.g];
					const double wg = wrow[r.g];
					// the next gate of the pass (a later one: passes keep the sequential
					// order) continues this reduction when it has the same block and weight
					merged += qpt;
					bool flush = true;
					if (gi + 1 < pr.gend && merged + qpt <= HESS_MERGE)
					{
						const int g2 = a.W.gate[gi + 1].g;
						flush = (a.block[g2] != blk || wrow[g2] != wg);
					}
					for (unsigned q = threadIdx.x; q < (unsigned)Q; q += blockDim.x)
					{
						unsigned ex, ew, ey, ez;
						quartet(r, q, tpar, ex, ew, ey, ez);
						const T vx = tile[ex], vw = tile[ew], vy = tile[ey], vz = tile[ez];
						contract_quartet<P>(acc, dg[ex], dg[ew], dg[ey], dg[ez], vx, vw, vy, vz);
						if (apply)
						{
							T ox = P::madd2(G.k0, vx, G.k1, vw), ow = P::madd2(G.k2, vx, G.k3, vw);
							T oy = P::madd2(G.c0, vy, G.c1, vz), oz = P::madd2(G.c2, vy, G.c3, vz);
							if (cg)
							{
								// entry x of the block: output (x >> 1) & 1 of the center (x < 4) or
								// corner block gains input x & 1 of the same block
								const unsigned ein = x < 4 ? ((x & 1) ? ez : ey) : ((x & 1) ? ew : ex);
								const T c = cg[ein];
								if (x < 2) oy = P::add(oy, c);
								else if (x < 4) oz = P::add(oz, c);
								else if (x < 6) ox = P::add(ox, c);
								else ow = P::add(ow, c);
							}
							tile[ex] = ox; tile[ew] = ow; tile[ey] = oy; tile[ez] = oz;
						}
					}
					if (flush)
					{
						block_reduce8<P>(acc, s.red, hrow + (size_t)blk * 16, wg, nred);
#pragma unroll
						for (int e = 0; e < 8; e++) acc[e] = P::acc_zero();
						merged = 0;
					}
					else __syncthreads();
				}
				if (pp < a.W.npass - 1) tile_store<P>(tile, kt, s, nlb, sh, false);
				__syncthreads();
			}
		}
	}
}

// ------------------------------------------------------------------------------------
// small kernels: staging, reductions, symmetrisation
// ------------------------------------------------------------------------------------

// dense target U (row-major 2^L x 2^L, FP64) -> -conj(U e_b) on b's sector, [b - b0][S]
template <class P>
__global__ void k_dense_columns(const double2* __restrict__ U, int L, long b0, long b1, typename P::T* __restrict__ out)
{
	const long S = 1L << (L - 1), n = 1L << L;
	const long total = (b1 - b0) * S;
	for (long u = blockIdx.x * (long)blockDim.x + threadIdx.x; u < total; u += (long)gridDim.x * blockDim.x)
	{
		const long bi = u / S, c = u - bi * S;
		const long b = b0 + bi;
		const int par = (__popcll(b) + __popcll(c)) & 1;
		const long arow = (c << 1) | par;
		const double2 v = U[arow * n + b];
		out[u] = P::make(-v.x, v.y);
	}
}

// host-supplied FP64 sector columns -> precision T
template <class P>
__global__ void k_convert(const double2* __restrict__ in, long n, typename P::T* __restrict__ out)
{
	for (long u = blockIdx.x * (long)blockDim.x + threadIdx.x; u < n; u += (long)gridDim.x * blockDim.x)
		out[u] = P::make(in[u].x, in[u].y);
}

// out[r] = sum over parts (fixed order) of part[c * len + r]
__global__ void k_sum_parts(const double* __restrict__ part, int nparts, long len, double* __restrict__ out)
{
	for (long r = blockIdx.x * (long)blockDim.x + threadIdx.x; r < len; r += (long)gridDim.x * blockDim.x)
	{
		double s = 0;
		for (int c = 0; c < nparts; c++) s += part[(size_t)c * len + r];
		out[r] = s;
	}
}

// per-gate gradients [ngates][16] -> per-block sums [nblocks][16], gates in order
__global__ void k_block_sum(const double* __restrict__ g, const int* __restrict__ block, int ngates, int nblocks, double* __restrict__ out)
{
	const int t = blockIdx.x * blockDim.x + threadIdx.x;
	if (t >= nblocks * 16) return;
	const int blk = t / 16, v = t % 16;
	double s = 0;
	for (int q = 0; q < ngates; q++) if (block[q] == blk) s += g[q * 16 + v];
	out[t] = s;
}

// diagonal blocks A -> A + A^T, then (second kernel) lower blocks mirrored from upper
__global__ void k_symm_diag(int nb, double2* __restrict__ h)
{
	const int m = nb * 8;
	for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < m * m; q += gridDim.x * blockDim.x)
	{
		const int r = q / m, c = q % m;
		if (r / 8 != c / 8) continue;
		if (c % 8 < r % 8)
		{
			const double2 a = h[(long)r * m + c], b = h[(long)c * m + r];
			const double2 s = make_double2(a.x + b.x, a.y + b.y);
			h[(long)r * m + c] = s; h[(long)c * m + r] = s;
		}
		else if (c % 8 == r % 8) { h[(long)r * m + c].x *= 2; h[(long)r * m + c].y *= 2; }
	}
}

__global__ void k_mirror(int nb, double2* __restrict__ h)
{
	const int m = nb * 8;
	for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < m * m; q += gridDim.x * blockDim.x)
	{
		const int r = q / m, c = q % m;
		if (c / 8 < r / 8) h[(long)r * m + c] = h[(long)c * m + r];
	}
}

int grid_cap(long work, int threads)
{
	long b = (work + threads - 1) / threads;
	const long cap = (long)mgcu_ctx()->nsm * 8;
	return (int)std::max(1L, std::min(b, cap));
}

}  // namespace

// ======================================================================================
// targets
// ======================================================================================
struct TargetProg
{
	int kt = -1, prec = -1, threads = -1;
	int max_pm = MAXPM;            // most distinct matrices any pass stages
	bool wcons = false;            // every gate conserves the Hamming weight (k_target_w applies)
	int max_g = MAXPG;             // most gates in one pass
	Sched sched;
	DevBuf pass, gate, mats, kinds, tg, pm, pmats;
};

// Exact classification of a 2x2 block (entries row-major); for BK_RI the entries are
// stored as (c_re, c_im) coefficients of the possibly swapped components of the input:
// real a -> (a, a), imaginary i b -> (-b, b) with the swap bit set.
static int classify_block(const mgc* e, unsigned& rot, mgc* stored)
{
	auto is = [](mgc z, double re, double im) { return z.re == re && z.im == im; };
	for (int q = 0; q < 4; q++) stored[q] = e[q];
	rot = 0;
	const bool offz = is(e[1], 0, 0) && is(e[2], 0, 0), diagz = is(e[0], 0, 0) && is(e[3], 0, 0);
	if (offz && is(e[0], 1, 0) && is(e[3], 1, 0)) return BK_ID;
	if (diagz && is(e[1], 1, 0) && is(e[2], 1, 0)) return BK_SWAP;
	if (offz && is(e[0], 1, 0) && is(e[3], -1, 0)) return BK_NEG1;
	if (offz && is(e[0], 1, 0)) return BK_D1;
	if (offz) return BK_DIAG;
	if (diagz) return BK_ANTI;
	bool ri = true;
	for (int q = 0; q < 4; q++) ri = ri && (e[q].re == 0 || e[q].im == 0);
	if (!ri) return BK_GEN;
	for (int q = 0; q < 4; q++)
	{
		if (e[q].re == 0 && e[q].im != 0) { rot |= 1u << q; stored[q] = mgc_make(-e[q].im, e[q].im); }
		else stored[q] = mgc_make(e[q].re, e[q].re);
	}
	return BK_RI;
}

// 1 for a block [[c, i s], [i s, c]] with c, s real (a hopping term): BK_RI with real
// diagonal and imaginary off-diagonal entries, equal in pairs
static int sym_hop(int kind, unsigned rot, const mgc* e)
{
	return kind == BK_RI && rot == 6u && e[0].re == e[3].re && e[1].im == e[2].im;
}

template <class P>
static int upload_target_mats(const mgg* gates, int ng, DevBuf& buf, DevBuf& kinds, std::vector<int>& k)
{
	typedef typename P::T T;
	std::vector<T> h((size_t)std::max(ng, 1) * 8);
	k.assign((size_t)std::max(ng, 1), 0);
	for (int g = 0; g < ng; g++)
	{
		mgc sc[4], sk[4];
		unsigned rc, rk;
		const int kc = classify_block(gates[g].c, rc, sc), kk = classify_block(gates[g].k, rk, sk);
		k[g] = kc | (kk << 3) | (int)(rc << 6) | (int)(rk << 10) | (sym_hop(kc, rc, gates[g].c) << 14)
			| (sym_hop(kk, rk, gates[g].k) << 15);
		for (int q = 0; q < 4; q++)
		{
			h[(size_t)g * 8 + q] = P::make(sc[q].re, sc[q].im);
			h[(size_t)g * 8 + 4 + q] = P::make(sk[q].re, sk[q].im);
		}
	}
	int e = buf.alloc(sizeof(T) * h.size());
	if (!e) e = kinds.alloc(sizeof(int) * k.size());
	if (e) return e;
	cudaStream_t st = mgcu_stream();
	MGCU_TRY(cudaMemcpyAsync(buf.p, h.data(), sizeof(T) * h.size(), cudaMemcpyHostToDevice, st));
	MGCU_TRY(cudaMemcpyAsync(kinds.p, k.data(), sizeof(int) * k.size(), cudaMemcpyHostToDevice, st));
	MGCU_TRY(cudaStreamSynchronize(st));
	return 0;
}

struct mgcu_target
{
	int L;
	int kind;                      // 0 circuit, 1 dense
	std::vector<mgg> gates;
	std::vector<int> wires;
	DevBuf dense;                  // FP64 U on the device
	TargetProg progs[3];           // per precision
	int resident = 0;
	DevBuf res_cols[3];            // resident -conj(U e_b) per precision
	int res_kt[3] = { -1, -1, -1 };
	bool res_valid[3] = { false, false, false };
	// the gate list the target sweep runs (fermionic swaps relabelled away, see
	// relabel_fswaps) with per-gate Jordan-Wigner string wires
	int tuned_kt[3][32] = {};      // batch tile choice per precision and L (0: not tuned yet)
	std::map<std::array<int, 4>, std::array<int, 2>> tuned_sweep;   // plan sweep choice: (prec, tile bits, weight-restricted, 0) -> (threads, quartets)
	bool sweep_ready = false;
	std::vector<mgg> sg;
	std::vector<int> sw;
	std::vector<unsigned> smask;
};

// Remove fermionic swaps (center [[0,1],[1,0]], corner diag(1,-1)) from a circuit
// exactly.  An fswap on wires (X, Y) is a SWAP, absorbed by relabelling the logical
// wires of all later gates, times CZ(X, Y).  Each pending CZ is moved past the later
// gates: a gate on both of its wires absorbs it (corner block times diag(1,-1) on the
// right); a gate on one of them, (X, u) with the CZ on (X, v), becomes the gate with
// its off-diagonal entries negated when wire v is 1 (v joins the gate's string);
// other gates commute with it.  Applies only when the relabelling ends at the identity
// (true for fswap networks that restore the qubit order, such as Jordan-Wigner hops);
// CZs still pending at the end are appended as gates.  Returns false (and leaves the
// outputs empty) when the circuit has no fswap or the order is not restored.
static bool relabel_fswaps(int L, const std::vector<mgg>& gates, const std::vector<int>& wires,
	std::vector<mgg>& og, std::vector<int>& ow, std::vector<unsigned>& om)
{
	auto is = [](mgc z, double re, double im) { return z.re == re && z.im == im; };
	auto fswap = [&](const mgg& g) {
		return is(g.c[0], 0, 0) && is(g.c[1], 1, 0) && is(g.c[2], 1, 0) && is(g.c[3], 0, 0)
			&& is(g.k[0], 1, 0) && is(g.k[1], 0, 0) && is(g.k[2], 0, 0) && is(g.k[3], -1, 0);
	};
	og.clear(); ow.clear(); om.clear();
	bool any = false;
	for (const mgg& g : gates) any = any || fswap(g);
	if (!any || L > 32) return false;
	std::vector<int> pi(L);
	for (int q = 0; q < L; q++) pi[q] = q;
	std::vector<std::pair<int, int>> cz;   // pending CZs on physical wires (u < v)
	for (size_t i = 0; i < gates.size(); i++)
	{
		const int X = pi[wires[2 * i]], Y = pi[wires[2 * i + 1]];
		if (fswap(gates[i]))
		{
			const std::pair<int, int> c(std::min(X, Y), std::max(X, Y));
			auto it = std::find(cz.begin(), cz.end(), c);
			if (it != cz.end()) cz.erase(it); else cz.push_back(c);
			std::swap(pi[wires[2 * i]], pi[wires[2 * i + 1]]);
			continue;
		}
		mgg g = gates[i];
		unsigned mask = 0;
		for (size_t j = 0; j < cz.size();)
		{
			const int u = cz[j].first, v = cz[j].second;
			const bool hu = (u == X || u == Y), hv = (v == X || v == Y);
			if (hu && hv)
			{
				g.k[1] = mgc_make(-g.k[1].re, -g.k[1].im);
				g.k[3] = mgc_make(-g.k[3].re, -g.k[3].im);
				cz.erase(cz.begin() + j);
				continue;
			}
			if (hu) mask ^= 1u << v;
			else if (hv) mask ^= 1u << u;
			j++;
		}
		og.push_back(g); ow.push_back(X); ow.push_back(Y); om.push_back(mask);
	}
	for (int q = 0; q < L; q++)
		if (pi[q] != q) { og.clear(); ow.clear(); om.clear(); return false; }
	for (const auto& c : cz)
	{
		mgg g;
		for (int q = 0; q < 4; q++) { g.c[q] = mgc_make(q == 0 || q == 3 ? 1 : 0, 0); g.k[q] = mgc_make(0, 0); }
		g.k[0] = mgc_make(1, 0); g.k[3] = mgc_make(-1, 0);
		og.push_back(g); ow.push_back(c.first); ow.push_back(c.second); om.push_back(0);
	}
	return true;
}

static void prepare_sweep(mgcu_target* t)
{
	if (t->sweep_ready) return;
	if (!relabel_fswaps(t->L, t->gates, t->wires, t->sg, t->sw, t->smask))
	{
		t->sg = t->gates; t->sw = t->wires;
		t->smask.assign(t->gates.size(), 0u);
	}
	t->sweep_ready = true;
}

template <class P>
static int upload_mats(const mgg* gates, int ng, DevBuf& buf)
{
	typedef typename P::T T;
	std::vector<T> h((size_t)std::max(ng, 1) * 8);
	for (int g = 0; g < ng; g++)
		for (int q = 0; q < 4; q++)
		{
			h[(size_t)g * 8 + q] = P::make(gates[g].c[q].re, gates[g].c[q].im);
			h[(size_t)g * 8 + 4 + q] = P::make(gates[g].k[q].re, gates[g].k[q].im);
		}
	int e = buf.alloc(sizeof(T) * h.size());
	if (e) return e;
	MGCU_TRY(cudaMemcpyAsync(buf.p, h.data(), sizeof(T) * h.size(), cudaMemcpyHostToDevice, mgcu_stream()));
	MGCU_TRY(cudaStreamSynchronize(mgcu_stream()));
	return 0;
}

// the 2x2 block inverses of the gates (k_columns_adj); 1 when every block is invertible with
// |det| at least 1e-8 of its largest entry squared, 0 otherwise (nothing uploaded then)
template <class P>
static int upload_inverses(const mgg* gates, int ng, DevBuf& buf, bool& ok)
{
	typedef typename P::T T;
	std::vector<T> h((size_t)std::max(ng, 1) * 8);
	ok = true;
	auto inv = [&](const mgc* e, T* out) {
		const mgc det = mgc_sub(mgc_mul(e[0], e[3]), mgc_mul(e[1], e[2]));
		double mx = 0;
		for (int q = 0; q < 4; q++) mx = std::max(mx, std::hypot(e[q].re, e[q].im));
		const double d2 = det.re * det.re + det.im * det.im;
		if (!(std::sqrt(d2) >= 1e-8 * mx * mx) || mx == 0) { ok = false; return; }
		const mgc id = mgc_make(det.re / d2, -det.im / d2);   // 1 / det
		const mgc r[4] = { mgc_mul(e[3], id), mgc_mul(mgc_make(-e[1].re, -e[1].im), id),
			mgc_mul(mgc_make(-e[2].re, -e[2].im), id), mgc_mul(e[0], id) };
		for (int q = 0; q < 4; q++) out[q] = P::make(r[q].re, r[q].im);
	};
	for (int g = 0; g < ng && ok; g++)
	{
		inv(gates[g].c, &h[(size_t)g * 8]);
		inv(gates[g].k, &h[(size_t)g * 8 + 4]);
	}
	if (!ok) return 0;
	int e = buf.alloc(sizeof(T) * h.size());
	if (e) return e;
	MGCU_TRY(cudaMemcpyAsync(buf.p, h.data(), sizeof(T) * h.size(), cudaMemcpyHostToDevice, mgcu_stream()));
	MGCU_TRY(cudaStreamSynchronize(mgcu_stream()));
	return 0;
}

static int upload_sched(const Sched& s, DevBuf& pass, DevBuf& gate)
{
	cudaStream_t st = mgcu_stream();
	int e = pass.alloc(sizeof(PassRec) * std::max<size_t>(s.pass.size(), 1));
	if (e) return e;
	e = gate.alloc(sizeof(GateRec) * std::max<size_t>(s.gate.size(), 1));
	if (e) return e;
	MGCU_TRY(cudaMemcpyAsync(pass.p, s.pass.data(), sizeof(PassRec) * s.pass.size(), cudaMemcpyHostToDevice, st));
	if (!s.gate.empty()) MGCU_TRY(cudaMemcpyAsync(gate.p, s.gate.data(), sizeof(GateRec) * s.gate.size(), cudaMemcpyHostToDevice, st));
	MGCU_TRY(cudaStreamSynchronize(st));
	return 0;
}

// TGate.act of a gate (type as in GateRec, kinds of its center and corner block): the
// range of rho = r - (|b| - popc(nlb)) for which the gate changes a nonzero amplitude of a
// column of weight |b|.  A member of popcount offset o (over r) is nonzero when
// rho + o is -1 or 0; gates on the dropped qubit pair their members by the parity of the
// quartet's base, which equals the parity of rho.
static int weight_act(int type, int kc, int kk)
{
	auto live = [](int rho, int o) { return rho + o == -1 || rho + o == 0; };
	auto changes = [&](int kind, int rho, int oa, int ob) {
		if (kind == BK_ID) return false;
		if (kind == BK_D1 || kind == BK_NEG1) return live(rho, ob);   // only the second member moves
		return live(rho, oa) || live(rho, ob);
	};
	int lo = 99, hi = -99;
	for (int rho = -3; rho <= 0; rho++)
	{
		const int sp = rho & 1;
		int ox, ow, oy, oz;   // popcount offsets of x, w (corner pair) and y, z (center pair)
		if (type == 0) { ox = 0; ow = 2; oy = 1; oz = 1; }
		else if (type == 1) { if (!sp) { ox = 0; ow = 1; oy = 1; oz = 2; } else { ox = 1; ow = 2; oy = 0; oz = 1; } }
		else { if (!sp) { ox = 0; ow = 1; oy = 2; oz = 1; } else { ox = 1; ow = 2; oy = 1; oz = 0; } }
		if (changes(kk, rho, ox, ow) || changes(kc, rho, oy, oz)) { lo = std::min(lo, rho); hi = std::max(hi, rho); }
	}
	return lo <= hi ? (0x100 | (lo + 4) | (hi + 4) << 4) : 0;
}

template <class P>
static int build_target_prog(mgcu_target* t, int kt, int threads, TargetProg& tp)
{
	{
		typedef typename P::T T;
		prepare_sweep(t);
		const std::vector<mgg>& gates = t->sg;
		schedule(t->L, kt, t->sw.data(), (int)gates.size(), true, tp.sched, sizeof(T) >= 16 ? 1 : 2, t->smask.data());
		// distinct matrices, then passes split so that each stages at most MAXPM of them
		const int ngt = (int)gates.size();
		std::vector<int> uid(std::max(ngt, 1), 0);
		{
			std::map<std::array<double, 16>, int> seen;
			for (int g = 0; g < ngt; g++)
			{
				std::array<double, 16> key;
				memcpy(key.data(), &gates[g], sizeof(key));
				auto it = seen.emplace(key, (int)seen.size()).first;
				uid[g] = it->second;
			}
		}
		std::vector<int> slot(std::max<size_t>(tp.sched.gate.size(), 1), 0);
		std::vector<int2> pmh;
		std::vector<int> pm_first;   // first-use matrix per staged slot, all passes
		{
			Sched split;
			split.pass_of = tp.sched.pass_of;
			split.gate = tp.sched.gate;
			for (const PassRec& pr : tp.sched.pass)
			{
				int gb = pr.gbeg;
				while (gb < pr.gend || gb == pr.gbeg)
				{
					std::map<int, int> loc;
					const int off = (int)pm_first.size();
					int ge = gb;
					for (; ge < pr.gend && ge - gb < MAXPG; ge++)
					{
						const int u = uid[tp.sched.gate[ge].g];
						auto it = loc.find(u);
						if (it == loc.end())
						{
							if ((int)loc.size() == MAXPM) break;
							it = loc.emplace(u, (int)loc.size()).first;
							pm_first.push_back(tp.sched.gate[ge].g);
						}
						slot[ge] = it->second;
					}
					PassRec q = pr;
					q.gbeg = gb; q.gend = ge;
					split.pass.push_back(q);
					pmh.push_back(make_int2(off * 8, (int)loc.size()));
					if (ge == gb) break;   // empty pass
					gb = ge;
				}
			}
			tp.sched.pass.swap(split.pass);
		}
		tp.max_pm = 1;
		for (const int2& v : pmh) tp.max_pm = std::max(tp.max_pm, v.y);
		tp.max_g = 1;
		for (const PassRec& q : tp.sched.pass) tp.max_g = std::max(tp.max_g, q.gend - q.gbeg);
		int e = upload_sched(tp.sched, tp.pass, tp.gate);
		if (e) return e;
		std::vector<int> kw;
		e = upload_target_mats<P>(gates.data(), ngt, tp.mats, tp.kinds, kw);
		if (e) return e;
		// k_target's records; the auxiliary bit of a gate on the dropped qubit is a high
		// tile bit, away from the swizzle's two conflicting low pairs
		constexpr unsigned ES = sizeof(typename P::T);
		auto ins0 = [](unsigned v, int pos) { return ((v >> pos) << (pos + 1)) | (v & ((1u << pos) - 1u)); };
		std::vector<TGate> tg(std::max<size_t>(tp.sched.gate.size(), 1));
		memset(tg.data(), 0, sizeof(TGate) * tg.size());
		std::vector<int> pass_of_rec(tp.sched.gate.size(), 0);
		for (size_t p = 0; p < tp.sched.pass.size(); p++)
			for (int i = tp.sched.pass[p].gbeg; i < tp.sched.pass[p].gend; i++) pass_of_rec[i] = (int)p;
		for (size_t i = 0; i < tp.sched.gate.size(); i++)
		{
			const GateRec& r = tp.sched.gate[i];
			const PassRec& pr = tp.sched.pass[pass_of_rec[i]];
			// the gate's string split into local positions, nonlocal compact bits and the
			// dropped qubit
			unsigned ml = 0, mnl = 0, md = 0;
			for (int q = 0; q < t->L; q++)
			{
				if (!(t->smask[r.g] & (1u << q))) continue;
				if (q == t->L - 1) { md = 1; continue; }
				const int cbit = t->L - 2 - q;
				int lp = -1;
				for (int j = 0; j < kt; j++) if (pr.lbits[j] == cbit) lp = j;
				if (lp >= 0) ml |= 1u << lp; else mnl |= 1u << cbit;
			}
			int pa, pb;
			if (r.type == 0) { pa = r.la; pb = r.lb; }
			else
			{
				// auxiliary bit: a high tile bit outside the gate's string
				pa = r.type == 1 ? r.la : r.lb;
				pb = -1;
				for (int j = kt - 1; j >= 0 && pb < 0; j--)
					if (j != pa && !(ml & (1u << j))) pb = j;
				if (pb < 0) { mg_set_error("no auxiliary tile bit outside a gate's string"); return MG_ERR_ARG; }
			}
			const int lo = std::min(pa, pb), hi = std::max(pa, pb);
			const unsigned SA = tsw<ES>(1u << pa) * ES, SB = tsw<ES>(1u << pb) * ES;
			TGate& o = tg[i];
			o.m.x = (int)(r.type == 0 ? (SA ^ SB) : SA);
			o.m.y = (int)(r.type == 2 ? (SA ^ SB) : SB);
			o.m.z = (int)(r.type == 0 ? SA : (r.type == 1 ? (SA ^ SB) : SB));
			o.m.w = (int)(r.type == 0 ? 0u : SB);
			unsigned d[3], dpar = 0, spar = 0;
			for (int k = 0; k < 3; k++)
			{
				const unsigned e = ins0(ins0((unsigned)threads << k, lo), hi);
				d[k] = tsw<ES>(e) * ES;
				const unsigned pe = (unsigned)(__builtin_popcount(e) & 1);
				dpar |= pe << k;
				spar |= ((unsigned)(__builtin_popcount(e & ml) & 1) ^ (md & pe)) << k;
			}
			o.h.x = lo | hi << 5 | (int)(dpar << 10) | kw[r.g] << 13;
			o.h.y = slot[i];
			o.h.z = (int)d[0]; o.h.w = (int)d[1]; o.d4 = (int)d[2];
			o.sl = (int)(ml | md << 16 | spar << 17);
			o.snl = (int)mnl;
			o.act = weight_act(r.type, kw[r.g] & 7, (kw[r.g] >> 3) & 7);
		}
		// the weight-restricted sweep applies when no corner block mixes |00> and |11>
		tp.wcons = true;
		for (size_t i = 0; i < tp.sched.gate.size(); i++)
		{
			const int kk = (kw[tp.sched.gate[i].g] >> 3) & 7;
			tp.wcons = tp.wcons && (kk == BK_ID || kk == BK_D1 || kk == BK_NEG1 || kk == BK_DIAG);
		}
		e = tp.tg.alloc(sizeof(TGate) * tg.size());
		if (e) return e;
		MGCU_TRY(cudaMemcpy(tp.tg.p, tg.data(), sizeof(TGate) * tg.size(), cudaMemcpyHostToDevice));
		// staged matrices: the classified entries of each slot's first gate
		std::vector<T> hm(std::max<size_t>(pm_first.size(), 1) * 8);
		for (size_t i = 0; i < pm_first.size(); i++)
		{
			mgc sc[4], sk[4];
			unsigned rc, rk;
			classify_block(gates[pm_first[i]].c, rc, sc);
			classify_block(gates[pm_first[i]].k, rk, sk);
			for (int q = 0; q < 4; q++)
			{
				hm[i * 8 + q] = P::make(sc[q].re, sc[q].im);
				hm[i * 8 + 4 + q] = P::make(sk[q].re, sk[q].im);
			}
		}
		e = tp.pmats.alloc(sizeof(T) * hm.size());
		if (!e) e = tp.pm.alloc(sizeof(int2) * std::max<size_t>(pmh.size(), 1));
		if (e) return e;
		MGCU_TRY(cudaMemcpy(tp.pmats.p, hm.data(), sizeof(T) * hm.size(), cudaMemcpyHostToDevice));
		MGCU_TRY(cudaMemcpy(tp.pm.p, pmh.data(), sizeof(int2) * pmh.size(), cudaMemcpyHostToDevice));
		tp.kt = kt;
		tp.threads = threads;
	}
	return 0;
}

// the target's cached program for this precision, rebuilt when the tile or block size changes
template <class P>
static int target_prog(mgcu_target* t, int kt, int threads, TargetProg*& out)
{
	TargetProg& tp = t->progs[P::kId];
	if (tp.kt != kt || tp.threads != threads)
	{
		const int e = build_target_prog<P>(t, kt, threads, tp);
		if (e) { tp.kt = -1; return e; }
	}
	out = &tp;
	return 0;
}

template <class P>
static int target_pm_cap(mgcu_target* t, int kt, int threads, int& cap, bool& wcons, int& maxg)
{
	TargetProg* tp = nullptr;
	const int e = target_prog<P>(t, kt, threads, tp);
	if (!e) { cap = tp->max_pm; wcons = tp->wcons; maxg = tp->max_g; }
	return e;
}

extern "C" mgcu_target* mgcu_target_circuit(const mgg* gates, const int* wires, int ngates, int L)
{
	if (!mgcu_ctx()) return nullptr;
	mgcu_target* t = new mgcu_target();
	t->L = L; t->kind = 0;
	t->gates.assign(gates, gates + ngates);
	t->wires.assign(wires, wires + 2 * ngates);
	return t;
}

extern "C" mgcu_target* mgcu_target_dense(const mgc* U, int L)
{
	if (!mgcu_ctx()) return nullptr;
	mgcu_target* t = new mgcu_target();
	t->L = L; t->kind = 1;
	const size_t n = (size_t)1 << L;
	if (t->dense.alloc(sizeof(double2) * n * n)) { delete t; return nullptr; }
	if (cudaMemcpy(t->dense.p, U, sizeof(double2) * n * n, cudaMemcpyHostToDevice) != cudaSuccess)
	{
		mg_set_error("copying a dense target to the GPU failed");
		delete t;
		return nullptr;
	}
	return t;
}

extern "C" void mgcu_target_destroy(mgcu_target* t) { delete t; }
extern "C" int mgcu_target_sweep_gates(mgcu_target* t)
{
	if (t->kind != 0) return -1;
	prepare_sweep(t);
	return (int)t->sg.size();
}

// 1 when every gate of the swept circuit conserves the Hamming weight (no corner block
// mixes |00> and |11>), so the GPU sweep visits only the amplitudes of the column's weight
extern "C" int mgcu_target_conserves_weight(mgcu_target* t)
{
	if (t->kind != 0) return 0;
	prepare_sweep(t);
	for (const mgg& g : t->sg)
	{
		unsigned rot;
		mgc st[4];
		const int kk = classify_block(g.k, rot, st);
		if (kk != BK_ID && kk != BK_D1 && kk != BK_NEG1 && kk != BK_DIAG) return 0;
	}
	return 1;
}
extern "C" int mgcu_target_L(const mgcu_target* t) { return t->L; }
extern "C" void mgcu_target_set_resident(mgcu_target* t, int enable)
{
	t->resident = enable;
	if (!enable)
		for (int i = 0; i < 3; i++)
		{
			t->res_valid[i] = false;
			t->res_cols[i].release();
		}
}
// 1 when the target keeps its columns resident, 0 when not, -1 for a dense target (whose
// columns are never swept)
extern "C" int mgcu_target_resident(const mgcu_target* t) { return t->kind == 0 ? t->resident : -1; }

extern "C" int mgcu_target_apply(mgcu_target* t, const mgc* psi, mgc* out)
{
	if (t->kind == 0)
		return mgcu_circuit_forward(t->gates.data(), t->wires.data(), (int)t->gates.size(), t->L, psi, nullptr, out);
	// dense: out = U psi (FP64 matrix-vector product on the GPU)
	return mgcu_dense_matvec(t->dense.p, t->L, psi, out);
}

// ======================================================================================
// plans
// ======================================================================================
struct mgcu_plan
{
	mgcu_plan_desc d;
	std::vector<int> wires, block, place;
	std::vector<double> place_w;
	int L, nb, kt, threads, grid_a, grid_b, grid_t, prec;
	int kt_t, threads_t, nc_t;     // k_target's tile bits, block size and columns per block
	size_t smem_t;                 // k_target: its tile, tables, scratch and pm_cap staged matrices
	int pm_cap = MAXPM;            // staged matrices per pass k_target has room for
	bool w_t = false;              // the weight-restricted sweep (k_target_w)
	int maxg_t = MAXPG;            // k_target_w: room for this many staged gate records
	int nq_t = 2;                  // k_target_w: live quartets per thread and iteration
	bool ktime = false;            // record events around k_target launches (mgcu_plan_time_ms)
	std::vector<cudaEvent_t> kev;  // start/stop pairs
	size_t kev_used = 0;
	~mgcu_plan() { for (cudaEvent_t ev : kev) cudaEventDestroy(ev); }
	long S;
	size_t tsize;
	size_t smem;
	long chunk;
	Sched ws;
	DevBuf d_pass, d_gate, d_mats, d_pass_of, d_block, d_place, d_placew;
	bool adj = false;              // gradient plan: checkpointed backward sweep (k_columns_adj)
	bool hgroup = false;           // Hessian plan: one item per (column, block, entry), see k_hessian
	bool adj_ok = false;           // the current gates are invertible (else the cached sweep)
	DevBuf d_mats_inv, ck;
	DevBuf su, sw, sh, cache, dcache, part_f, part_g, part_h, cols64, cols;
	DevBuf out_f, out_g, out_blk, out_h, flush;
	int nparts_h;
};

static size_t prec_tsize(int prec) { return prec == MG_PREC_FP32_ID ? 8 : 16; }

// k_target's dynamic shared memory for tt threads: tile(s), deposit tables, reduction
// scratch, the staged matrices and (weight-restricted sweep) its tables and records
static size_t target_smem_bytes(const mgcu_plan* p, int tt)
{
	return (size_t)p->nc_t * ((size_t)1 << p->kt_t) * p->tsize + 2 * 128 * sizeof(unsigned)
		+ std::max<size_t>((size_t)(tt / 32) * 16 * sizeof(double), 16 * 16) + (size_t)p->pm_cap * 8 * p->tsize
		+ (p->w_t ? wtab_bytes(p->kt_t, p->maxg_t) : 0);
}

// -conj(U e_b) of a circuit target for b in [b0, b1) into out[b - b0]
template <class P>
static int launch_target(mgcu_plan* p, long b0, long b1, typename P::T* out)
{
	typedef typename P::T T;
	MgcuContext* c = mgcu_ctx();
	Args<P> a;
	memset(&a, 0, sizeof(a));
	a.L = p->L; a.nb = p->nb; a.kt = p->kt_t; a.S = p->S;
	TargetProg* tp = nullptr;
	int e = target_prog<P>(p->d.target, p->kt_t, p->threads_t, tp);
	if (e) return e;
	a.U.pass = tp->pass.as<PassRec>(); a.U.gate = tp->gate.as<GateRec>(); a.U.npass = (int)tp->sched.pass.size();
	a.um = tp->mats.as<T>();
	a.utg = tp->tg.as<TGate>();
	a.upm = tp->pm.as<int2>();
	a.upmats = tp->pmats.as<T>();
	if (tp->max_pm > p->pm_cap) { mg_set_error("target program stages %d matrices per pass, room for %d", tp->max_pm, p->pm_cap); return MG_ERR_ARG; }
	if (p->w_t && tp->max_g > p->maxg_t) { mg_set_error("target pass has %d gates, room for %d", tp->max_g, p->maxg_t); return MG_ERR_ARG; }
	const size_t wtab = p->w_t ? wtab_bytes(p->kt_t, p->maxg_t) : 0;
	a.pm_off = (unsigned)(p->smem_t - wtab - (size_t)p->pm_cap * 8 * p->tsize);
	a.wperm_off = (unsigned)(p->smem_t - wtab);
	a.b0 = b0; a.b1 = b1;
	a.ucols = out;
	const int grid = (int)std::min<long>(p->grid_t, p->nc_t == 2 ? std::max(1L, (b1 - b0 + 1) / 2) : b1 - b0);
	if (p->ktime)
		while (p->kev.size() < p->kev_used + 2)
		{
			cudaEvent_t ev;
			MGCU_TRY(cudaEventCreate(&ev));
			p->kev.push_back(ev);
		}
	if (p->ktime) MGCU_TRY(cudaEventRecord(p->kev[p->kev_used], mgcu_stream()));
	void (*kern)(Args<P>) = p->w_t ? w_kernel<P>(p->threads_t, p->nq_t) : target_kernel<P>(p->kt_t, p->threads_t, p->nc_t);
	if (!kern) { mg_set_error("no target-sweep kernel for 2^%d amplitudes and %d threads", p->kt_t, p->threads_t); return MG_ERR_ARG; }
	kern<<<grid, p->threads_t, p->smem_t, mgcu_stream()>>>(a);
	MGCU_LAUNCHED();
	if (p->ktime) { MGCU_TRY(cudaEventRecord(p->kev[p->kev_used + 1], mgcu_stream())); p->kev_used += 2; }
	return 0;
}

// f, gradients (and Hessian items) for columns [b0, b1) whose -conj(U e_b) are in dense
template <class P>
static int launch_columns(mgcu_plan* p, long b0, long b1, const typename P::T* dense, long dense_b0)
{
	typedef typename P::T T;
	MgcuContext* c = mgcu_ctx();
	Args<P> a;
	memset(&a, 0, sizeof(a));
	a.L = p->L; a.nb = p->nb; a.kt = p->kt; a.S = p->S;
	a.W.pass = p->d_pass.as<PassRec>(); a.W.gate = p->d_gate.as<GateRec>(); a.W.npass = (int)p->ws.pass.size();
	a.wm = p->d_mats.as<T>();
	a.ngates = p->d.ngates;
	a.dense = dense; a.dense_b0 = dense_b0;
	a.b0 = b0; a.b1 = b1;
	a.su = p->su.as<T>(); a.sw = p->sw.as<T>();
	a.cache = p->cache.as<T>();
	a.dcache = p->d.want_hess ? p->dcache.as<T>() : nullptr;
	a.cache_per_column = p->d.want_hess ? 1 : 0;
	a.want_grad = p->d.want_grad || p->d.want_hess;
	a.part_f = p->part_f.as<double>();
	a.part_g = p->part_g.as<double>();
	if (!a.want_grad) a.cache = nullptr;
	const long ncols = b1 - b0;
	const int grid = (int)std::min<long>(p->grid_a, ncols);
	if (p->adj && p->adj_ok)
	{
		a.wmi = p->d_mats_inv.as<T>();
		a.ck = p->ck.as<T>();
		k_columns_adj<P><<<grid, ADJ_THREADS, p->smem, mgcu_stream()>>>(a);
		MGCU_LAUNCHED();
		return 0;
	}
	if (p->adj)
	{
		// gates that are not invertible: the cached sweep, its cache allocated on first need
		const int e = p->cache.alloc((size_t)p->S * p->tsize * std::max(p->d.ngates, 1) * p->grid_a);
		if (e) return e;
		a.cache = p->cache.as<T>();
	}
	k_columns<P, false><<<grid, p->threads, p->smem, mgcu_stream()>>>(a);
	MGCU_LAUNCHED();
	if (p->d.want_hess)
	{
		a.place = p->d_place.as<int>(); a.place_w = p->d_placew.as<double>(); a.pass_of = p->d_pass_of.as<int>();
		a.block = p->d_block.as<int>(); a.nplace = p->d.nplace; a.mdim = 8 * p->d.nblocks; a.hgroup = p->hgroup ? 1 : 0;
		a.part_h = p->part_h.as<double>(); a.sh = p->sh.as<T>();
		const long nitems = ncols * p->d.nplace * 8;
		const int gb = (int)std::min<long>(p->grid_b, nitems);
		k_hessian<P><<<gb, p->threads, p->smem, mgcu_stream()>>>(a, nitems);
		MGCU_LAUNCHED();
	}
	return 0;
}

template <class P>
static int set_smem_attr()
{
	MgcuContext* c = mgcu_ctx();
	MGCU_TRY(cudaFuncSetAttribute(k_columns<P, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)std::min<size_t>(c->smem_optin, 227 * 1024)));
	MGCU_TRY(cudaFuncSetAttribute(k_columns_adj<P>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)std::min<size_t>(c->smem_optin, 227 * 1024)));
	void (*const tk[10])(Args<P>) = { k_target<P, 256, 4>, k_target<P, 256, 8>, k_target<P, 256, 0>, k_target<P, 512, 2>,
		k_target<P, 512, 4>, k_target<P, 512, 0>, k_target2<P, 4>, k_target2<P, 8>, k_target2<P, 0>, k_target<P, 128, 8> };
	for (auto k : tk) MGCU_TRY(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)std::min<size_t>(c->smem_optin, 227 * 1024)));
	void (*const wk[2])(Args<P>) = { k_target_w<P, 128, 2>, k_target_w<P, 256, 1> };
	for (auto k : wk) MGCU_TRY(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)std::min<size_t>(c->smem_optin, 227 * 1024)));
	MGCU_TRY(cudaFuncSetAttribute(k_hessian<P>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)std::min<size_t>(c->smem_optin, 227 * 1024)));
	return 0;
}

template <class P>
static int occupancy(int threads, size_t smem, int kt_t, int threads_t, int nc_t, size_t smem_t, bool w_t, int nq_t, bool adj, int& per_sm,
	int& per_sm_target)
{
	int n1 = 0, n2 = 0, n3 = 0;
	if (adj) MGCU_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n1, k_columns_adj<P>, ADJ_THREADS, smem));
	else MGCU_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n1, k_columns<P, false>, threads, smem));
	MGCU_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n2, k_hessian<P>, threads, smem));
	void (*kern)(Args<P>) = w_t ? w_kernel<P>(threads_t, nq_t) : target_kernel<P>(kt_t, threads_t, nc_t);
	if (!kern) { mg_set_error("no target-sweep kernel for 2^%d amplitudes and %d threads", kt_t, threads_t); return MG_ERR_ARG; }
	MGCU_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n3, kern, threads_t, smem_t));
	per_sm = std::max(1, adj ? n1 : std::min(n1, n2));   // gradient plans launch no Hessian items
	per_sm_target = std::max(1, n3);
	return 0;
}

// The target sweep's block size, chosen by timing: each candidate (threads, and for the
// weight-restricted sweep live quartets per thread and iteration) traces one resident wave
// of columns twice with the plan's own program, and the faster second run wins.  Every
// candidate applies the same operations to each amplitude in the same order, so the choice
// changes the speed only, never a bit of a result; it is cached on the target per
// precision, tile size and sweep kind.  The columns traced start at a third of the range,
// where the column weights are typical of the whole.
template <class P>
static int tune_target_sweep(mgcu_plan* p)
{
	typedef typename P::T T;
	MgcuContext* c = mgcu_ctx();
	mgcu_target* t = p->d.target;
	const std::array<int, 4> key = { p->prec, p->kt_t, p->w_t ? 1 : 0, 0 };
	std::vector<std::array<int, 2>> cand;
	auto it = t->tuned_sweep.find(key);
	if (it != t->tuned_sweep.end()) cand.push_back(it->second);
	else if (p->w_t) cand = { { 128, 2 }, { 256, 1 } };
	else
	{
		const int Q = 1 << (p->kt_t - 2);
		for (int th : { 128, 256, 512 })
		{
			const int q = Q / th;
			if (Q % th == 0 && ((th == 128 && q == 8) || (th == 256 && (q == 4 || q == 8)) || (th == 512 && (q == 2 || q == 4))))
				cand.push_back({ th, 2 });
		}
	}
	if (cand.empty()) return 0;
	int e = set_smem_attr<P>();
	if (e) return e;
	auto kernel_of = [&](const std::array<int, 2>& cd) {
		return p->w_t ? w_kernel<P>(cd[0], cd[1]) : target_kernel<P>(p->kt_t, cd[0], 1);
	};
	std::array<int, 2> best = cand[0];
	if (cand.size() > 1)
	{
		const long ncols = 1L << p->L;
		DevBuf tmp;
		if (tmp.alloc(sizeof(T) * (size_t)p->S * std::min<long>(ncols, (long)c->nsm * 4))) { cudaGetLastError(); return 0; }
		cudaEvent_t ev[2];
		MGCU_TRY(cudaEventCreate(&ev[0]));
		if (cudaEventCreate(&ev[1]) != cudaSuccess) { cudaEventDestroy(ev[0]); return MG_ERR_DEVICE; }
		float best_ms = -1;
		for (const auto& cd : cand)
		{
			int per = 0;
			const size_t sm = target_smem_bytes(p, cd[0]);
			if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel_of(cd), cd[0], sm) != cudaSuccess || per < 1) continue;
			p->threads_t = cd[0]; p->nq_t = cd[1]; p->smem_t = sm;
			p->grid_t = c->nsm * std::min(per, 4);
			const long n = std::min<long>(ncols, p->grid_t);
			const long b0 = std::min(((ncols / 3) & ~63L), ncols - n);
			float ms = -1;
			for (int rep = 0; rep < 2 && !e; rep++)
			{
				e = cudaEventRecord(ev[0], mgcu_stream()) != cudaSuccess ? MG_ERR_DEVICE : 0;
				if (!e) e = launch_target<P>(p, b0, b0 + n, tmp.as<T>());
				if (!e) e = cudaEventRecord(ev[1], mgcu_stream()) != cudaSuccess ? MG_ERR_DEVICE : 0;
				if (!e) e = cudaEventSynchronize(ev[1]) != cudaSuccess ? MG_ERR_DEVICE : 0;
				if (!e) cudaEventElapsedTime(&ms, ev[0], ev[1]);
			}
			if (e) break;
			if (best_ms < 0 || ms < best_ms) { best_ms = ms; best = cd; }
		}
		cudaEventDestroy(ev[0]);
		cudaEventDestroy(ev[1]);
		if (e) { mg_set_error("timing the target sweep's block sizes failed"); return e; }
		t->tuned_sweep[key] = best;
	}
	p->threads_t = best[0]; p->nq_t = best[1]; p->smem_t = target_smem_bytes(p, best[0]);
	return 0;
}

extern "C" mgcu_plan* mgcu_plan_create(const mgcu_plan_desc* d)
{
	MgcuContext* c = mgcu_ctx();
	if (!c) return nullptr;
	if (d->L < 3 || d->L > 30)
	{
		mg_set_error("batched evaluation supports 3 <= nqubits <= 30 (got %d)", d->L);
		return nullptr;
	}
	for (int g = 0; g < 2 * d->ngates; g++)
		if (d->wires[g] < 0 || d->wires[g] >= d->L || (g % 2 == 1 && d->wires[g] == d->wires[g - 1]))
		{
			mg_set_error("invalid wire pair for gate %d", g / 2);
			return nullptr;
		}
	mgcu_plan* p = new mgcu_plan();
	p->d = *d;
	p->wires.assign(d->wires, d->wires + 2 * d->ngates);
	p->block.resize(std::max(d->ngates, 1));
	for (int g = 0; g < d->ngates; g++) p->block[g] = d->block ? d->block[g] : g;
	if (d->want_hess)
	{
		p->place.assign(d->place, d->place + d->nplace);
		p->place_w.assign(d->place_w, d->place_w + (size_t)d->nplace * d->ngates);
		// the plain placements (every gate, unit weights on every later gate) of parameter
		// blocks shared by several gates become one grouped placement per block, at the
		// block's first gate (k_hessian's forward-mode items)
		const int ng = d->ngates;
		bool plain = d->nplace == ng && d->nblocks < ng && d->place && d->place_w && mgcu_option(MG_OPT_HESS_GROUP_ID) != 1;
		for (int q = 0; q < ng && plain; q++)
		{
			plain = d->place[q] == q;
			for (int l = 0; l < ng && plain; l++) plain = d->place_w[(size_t)q * ng + l] == (l > q ? 1.0 : 0.0);
		}
		if (plain)
		{
			std::vector<int> first(d->nblocks, -1);
			for (int g = 0; g < ng; g++)
				if (p->block[g] >= 0 && p->block[g] < d->nblocks && first[p->block[g]] < 0) first[p->block[g]] = g;
			p->place.clear();
			for (int b = 0; b < d->nblocks; b++) if (first[b] >= 0) p->place.push_back(first[b]);
			std::sort(p->place.begin(), p->place.end());
			p->place_w.assign(p->place.size() * (size_t)ng, 0.0);
			for (size_t q = 0; q < p->place.size(); q++)
				for (int l = p->place[q] + 1; l < ng; l++) p->place_w[q * ng + l] = 1.0;
			p->d.nplace = (int)p->place.size();
			p->hgroup = true;
		}
	}
	p->d.wires = p->wires.data(); p->d.block = p->block.data();
	p->d.place = p->place.data(); p->d.place_w = p->place_w.data();
	p->L = d->L; p->nb = d->L - 1; p->S = 1L << (d->L - 1);
	p->prec = d->precision;
	p->tsize = prec_tsize(p->prec);

	// gradient plans: the checkpointed sweep (k_columns_adj, no per-gate cache) when
	// FIT_CACHE = 2 asks for it (memory: one state per pass and block instead of one per gate);
	// otherwise the cache, which measured faster in float-float (L=16, 40 gates: 1.29 s against
	// 1.58 s per evaluation; L=18, 63 gates, even with the cache's grid cap: 1.43 s against
	// 1.79 s per 4096 columns): the inverses add a third to the backward sweep's arithmetic,
	// and the float-float sweeps are arithmetic-bound more than bound by the cache reads
	p->adj = d->want_grad && !d->want_hess && mgcu_option(MG_OPT_FIT_CACHE_ID) == 2;
	// tile size: 64 KB of state by default (2^12 complex of 16 B, 2^13 of 8 B); two tiles of
	// 32 KB for the checkpointed sweep
	int kt = (p->tsize == 16) ? 12 : 13;
	if (p->adj) kt--;
	const long opt_kt = mgcu_option(MG_OPT_TILE_BITS_ID);
	if (opt_kt > 0) kt = (int)opt_kt;
	kt = std::max(5, std::min(kt, MAXKT));   // >= 5: any gate fits beside the 3 fixed low bits
	while (kt > 5 && ((size_t)(p->adj ? 2 : 1) << kt) * p->tsize > 200 * 1024) kt--;
	p->kt = std::min(kt, p->nb);
	const int Q = 1 << (p->kt - 2);
	int threads = std::max(32, std::min(256, Q));
	const long opt_thr = mgcu_option(MG_OPT_THREADS_ID);
	if (opt_thr > 0) threads = (int)std::max(32L, std::min(256L, (opt_thr / 32) * 32));
	p->threads = threads;
	// tile(s), deposit tables, reduction scratch (for the block size of the kernel that runs:
	// k_columns_adj always launches ADJ_THREADS threads, more than `threads` for small tiles)
	p->smem = ((size_t)(p->adj ? 2 : 1) << p->kt) * p->tsize + 2 * 128 * sizeof(unsigned)
		+ red_bytes(p->adj ? std::max(threads, ADJ_THREADS) : threads);

	schedule(p->L, p->kt, p->wires.data(), d->ngates, false, p->ws);

	// the target sweep's own tile and block size (circuit targets only): by default 64 KB of
	// state (as TILE_BITS), independent of the fitted circuit's tile (smaller for the
	// checkpointed gradient sweep)
	{
		int ktt = opt_kt > 0 ? (int)std::max(5L, std::min<long>(opt_kt, MAXKT)) : (p->tsize == 16 ? 12 : 13);
		const long o = mgcu_option(MG_OPT_TARGET_TILE_BITS_ID);
		if (o > 0) ktt = (int)std::max(5L, std::min<long>(o, MAXKT));
		while (ktt > 5 && ((size_t)1 << ktt) * p->tsize > 128 * 1024) ktt--;
		p->kt_t = std::min(ktt, p->nb);
		// 2^12 amplitudes of 16 B: 128 threads with eight quartets each, three blocks per SM
		// (measured at L=16: 0.460 s per 8192-column launch against 0.495 s with 256 x 4)
		int tt = std::max(32, std::min(256, 1 << (p->kt_t - 2)));
		if (p->tsize == 16 && p->kt_t == 12) tt = 128;
		const long ot = mgcu_option(MG_OPT_TARGET_THREADS_ID);
		if (ot > 0) tt = (int)std::max(32L, std::min(512L, (ot / 32) * 32));
		p->threads_t = tt;
		p->nc_t = (mgcu_option(MG_OPT_TARGET_COLUMNS_ID) == 2 && tt == 256) ? 2 : 1;
		// targets that conserve the Hamming weight run the weight-restricted sweep (128
		// threads, one column per block) unless TARGET_DENSE asks for the full one
		bool wcons = false;
		if (d->target && d->target->kind == 0 && p->nc_t == 1 && mgcu_option(MG_OPT_TARGET_DENSE_ID) == 0
			&& (ot <= 0 || tt == 128 || tt == 256))
		{
			int e = 0, mp = MAXPM, mg = MAXPG;
			if (p->prec == MG_PREC_FP64_ID) e = target_pm_cap<PrecD>(d->target, p->kt_t, 128, mp, wcons, mg);
			else if (p->prec == MG_PREC_FP32_ID) e = target_pm_cap<PrecF>(d->target, p->kt_t, 128, mp, wcons, mg);
			else e = target_pm_cap<PrecX>(d->target, p->kt_t, 128, mp, wcons, mg);
			if (e) { delete p; return nullptr; }
			if (wcons)
			{
				// 128 threads x two quartets, or 256 x one (TARGET_THREADS 256)
				p->threads_t = tt = (ot == 256 ? 256 : 128);
				p->nq_t = tt == 256 ? 1 : 2;
				p->pm_cap = mp; p->w_t = true; p->maxg_t = mg;
			}
		}
		// room for the staged matrices of the target's busiest pass (built here, cached on the target)
		if (d->target && d->target->kind == 0 && !p->w_t)
		{
			int e = 0, mp = MAXPM, mg = MAXPG;
			if (p->prec == MG_PREC_FP64_ID) e = target_pm_cap<PrecD>(d->target, p->kt_t, tt, mp, wcons, mg);
			else if (p->prec == MG_PREC_FP32_ID) e = target_pm_cap<PrecF>(d->target, p->kt_t, tt, mp, wcons, mg);
			else e = target_pm_cap<PrecX>(d->target, p->kt_t, tt, mp, wcons, mg);
			if (e) { delete p; return nullptr; }
			p->pm_cap = mp;
		}
		p->smem_t = target_smem_bytes(p, tt);
		// the block size by timing (MG_OPT_TARGET_TUNE: 0 = when the trace has at least 2^14
		// columns, 1 = never, 2 = always) unless TARGET_THREADS fixes it
		const long tune = mgcu_option(MG_OPT_TARGET_TUNE_ID);
		if (d->target && d->target->kind == 0 && ot <= 0 && p->nc_t == 1 && tune != 1 && (tune == 2 || d->L >= 14))
		{
			int e = 0;
			if (p->prec == MG_PREC_FP64_ID) e = tune_target_sweep<PrecD>(p);
			else if (p->prec == MG_PREC_FP32_ID) e = tune_target_sweep<PrecF>(p);
			else e = tune_target_sweep<PrecX>(p);
			if (e) { delete p; return nullptr; }
		}
	}
	int per_sm = 1, per_sm_t = 1, e = 0;
	if (p->prec == MG_PREC_FP64_ID) { e = set_smem_attr<PrecD>(); if (!e) e = occupancy<PrecD>(threads, p->smem, p->kt_t, p->threads_t, p->nc_t, p->smem_t, p->w_t, p->nq_t, p->adj, per_sm, per_sm_t); }
	else if (p->prec == MG_PREC_FP32_ID) { e = set_smem_attr<PrecF>(); if (!e) e = occupancy<PrecF>(threads, p->smem, p->kt_t, p->threads_t, p->nc_t, p->smem_t, p->w_t, p->nq_t, p->adj, per_sm, per_sm_t); }
	else { e = set_smem_attr<PrecX>(); if (!e) e = occupancy<PrecX>(threads, p->smem, p->kt_t, p->threads_t, p->nc_t, p->smem_t, p->w_t, p->nq_t, p->adj, per_sm, per_sm_t); }
	if (e) { delete p; return nullptr; }
	const long opt_cps = mgcu_option(MG_OPT_CTAS_PER_SM_ID);
	if (opt_cps > 0) per_sm = (int)std::min<long>(per_sm, opt_cps);
	long grid = (long)c->nsm * per_sm;
	const long ncols_total = 1L << d->L;
	const size_t col_bytes = (size_t)p->S * p->tsize;
	const int ng = std::max(d->ngates, 1);
	const bool grad = d->want_grad || d->want_hess;
	// gradient caches are per block: keep them within 32 GB
	if (grad && !d->want_hess)
	{
		const long cap = (long)((32ull << 30) / ((size_t)ng * col_bytes));
		grid = std::max(1L, std::min(grid, cap));
	}
	grid = std::min(grid, ncols_total);
	p->grid_a = (int)grid;
	p->grid_b = (int)((long)c->nsm * per_sm);
	p->grid_t = (int)((long)c->nsm * (opt_cps > 0 ? std::min<long>(per_sm_t, opt_cps) : per_sm_t));

	// columns per chunk: Hessian caches per column (<= 16 GB) or staged target columns (<= 8 GB)
	long chunk = ncols_total;
	if (d->want_hess) chunk = std::max(1L, std::min(chunk, (long)((16ull << 30) / (2ull * ng * col_bytes))));
	chunk = std::max(1L, std::min(chunk, (long)((8ull << 30) / (col_bytes + (size_t)p->S * 16))));
	const long opt_chunk = mgcu_option(MG_OPT_CHUNK_COLUMNS_ID);
	if (opt_chunk > 0) chunk = std::min(chunk, opt_chunk);
	p->chunk = chunk;

	// device buffers
	const int mdim = 8 * std::max(d->nblocks, 1);
	e = 0;
	if (!e) e = upload_sched(p->ws, p->d_pass, p->d_gate);
	if (!e) e = p->su.alloc(col_bytes * grid);
	if (!e) e = p->sw.alloc(col_bytes * grid);
	if (!e && grad && !p->adj) e = p->cache.alloc(col_bytes * ng * (d->want_hess ? chunk : grid));
	if (!e && p->adj) e = p->ck.alloc(col_bytes * p->ws.pass.size() * grid);
	if (!e && d->want_hess) e = p->dcache.alloc(col_bytes * ng * chunk);
	if (!e && d->want_hess) e = p->sh.alloc(col_bytes * p->grid_b);
	if (!e) e = p->part_f.alloc(sizeof(double) * 2 * grid);
	if (!e) e = p->part_g.alloc(sizeof(double) * 16 * ng * grid);
	if (!e && d->want_hess) e = p->part_h.alloc(sizeof(double) * 2 * (size_t)mdim * mdim * p->grid_b);
	if (!e) e = p->out_f.alloc(sizeof(double) * 2);
	if (!e) e = p->out_g.alloc(sizeof(double) * 16 * ng);
	if (!e) e = p->out_blk.alloc(sizeof(double) * 16 * std::max(d->nblocks, 1));
	if (!e && d->want_hess) e = p->out_h.alloc(sizeof(double) * 2 * (size_t)mdim * mdim);
	if (!e) e = p->d_block.alloc(sizeof(int) * ng);
	if (!e) e = p->d_pass_of.alloc(sizeof(int) * ng);
	if (!e) e = p->cols.alloc(col_bytes * chunk);
	if (!e && !d->target) e = p->cols64.alloc((size_t)p->S * 16 * chunk);
	if (!e && d->want_hess) e = p->d_place.alloc(sizeof(int) * std::max(p->d.nplace, 1));
	if (!e && d->want_hess) e = p->d_placew.alloc(sizeof(double) * std::max<size_t>((size_t)p->d.nplace * ng, 1));
	if (e) { delete p; return nullptr; }
	cudaStream_t st = mgcu_stream();
	bool ok = cudaMemcpyAsync(p->d_block.p, p->block.data(), sizeof(int) * ng, cudaMemcpyHostToDevice, st) == cudaSuccess;
	ok = ok && cudaMemcpyAsync(p->d_pass_of.p, p->ws.pass_of.data(), sizeof(int) * d->ngates, cudaMemcpyHostToDevice, st) == cudaSuccess;
	if (d->want_hess)
	{
		ok = ok && cudaMemcpyAsync(p->d_place.p, p->place.data(), sizeof(int) * p->d.nplace, cudaMemcpyHostToDevice, st) == cudaSuccess;
		ok = ok && cudaMemcpyAsync(p->d_placew.p, p->place_w.data(), sizeof(double) * p->place_w.size(), cudaMemcpyHostToDevice, st) == cudaSuccess;
	}
	ok = ok && cudaStreamSynchronize(st) == cudaSuccess;
	if (!ok) { mg_set_error("uploading an evaluation plan failed"); delete p; return nullptr; }
	return p;
}

extern "C" void mgcu_plan_destroy(mgcu_plan* p) { delete p; }

extern "C" long mgcu_plan_chunk_columns(const mgcu_plan* p) { return p->chunk; }

extern "C" int mgcu_plan_set_gates(mgcu_plan* p, const mgg* gates)
{
	int e;
	if (p->prec == MG_PREC_FP64_ID) e = upload_mats<PrecD>(gates, p->d.ngates, p->d_mats);
	else if (p->prec == MG_PREC_FP32_ID) e = upload_mats<PrecF>(gates, p->d.ngates, p->d_mats);
	else e = upload_mats<PrecX>(gates, p->d.ngates, p->d_mats);
	if (e || !p->adj) return e;
	if (p->prec == MG_PREC_FP32_ID) return upload_inverses<PrecF>(gates, p->d.ngates, p->d_mats_inv, p->adj_ok);
	return upload_inverses<PrecX>(gates, p->d.ngates, p->d_mats_inv, p->adj_ok);
}

extern "C" int mgcu_plan_begin(mgcu_plan* p)
{
	cudaStream_t st = mgcu_stream();
	MGCU_TRY(cudaMemsetAsync(p->part_f.p, 0, p->part_f.n, st));
	MGCU_TRY(cudaMemsetAsync(p->part_g.p, 0, p->part_g.n, st));
	if (p->d.want_hess) MGCU_TRY(cudaMemsetAsync(p->part_h.p, 0, p->part_h.n, st));
	return 0;
}

template <class P>
static int plan_columns_t(mgcu_plan* p, long b0, long b1, const mgc* host_cols)
{
	typedef typename P::T T;
	MgcuContext* c = mgcu_ctx();
	mgcu_target* t = p->d.target;
	for (long c0 = b0; c0 < b1; c0 += p->chunk)
	{
		const long c1 = std::min(b1, c0 + p->chunk);
		const long n = (c1 - c0) * p->S;
		const T* dense = nullptr;
		long dense_b0 = c0;
		if (!t)
		{
			MGCU_TRY(cudaMemcpyAsync(p->cols64.p, host_cols + (size_t)(c0 - b0) * p->S, sizeof(double2) * n, cudaMemcpyHostToDevice, mgcu_stream()));
			k_convert<P><<<grid_cap(n, 256), 256, 0, mgcu_stream()>>>(p->cols64.as<double2>(), n, p->cols.as<T>());
			MGCU_LAUNCHED();
			dense = p->cols.as<T>();
		}
		else if (t->kind == 1)
		{
			k_dense_columns<P><<<grid_cap(n, 256), 256, 0, mgcu_stream()>>>(t->dense.as<double2>(), p->L, c0, c1, p->cols.as<T>());
			MGCU_LAUNCHED();
			dense = p->cols.as<T>();
		}
		else if (t->resident)
		{
			const int id = P::kId;
			if (!t->res_valid[id] || t->res_kt[id] != p->kt)
			{
				const long N = 1L << p->L;
				int e = t->res_cols[id].alloc((size_t)N * p->S * sizeof(T));
				if (e) return e;
				e = launch_target<P>(p, 0, N, t->res_cols[id].as<T>());
				if (e) return e;
				t->res_valid[id] = true; t->res_kt[id] = p->kt;
			}
			dense = t->res_cols[id].as<T>();
			dense_b0 = 0;
		}
		else
		{
			int e = launch_target<P>(p, c0, c1, p->cols.as<T>());
			if (e) return e;
			dense = p->cols.as<T>();
		}
		int e = launch_columns<P>(p, c0, c1, dense, dense_b0);
		if (e) return e;
	}
	return 0;
}

extern "C" int mgcu_plan_columns(mgcu_plan* p, long b0, long b1, const mgc* host_cols)
{
	if (b1 <= b0) return 0;
	if (p->prec == MG_PREC_FP64_ID) return plan_columns_t<PrecD>(p, b0, b1, host_cols);
	if (p->prec == MG_PREC_FP32_ID) return plan_columns_t<PrecF>(p, b0, b1, host_cols);
	return plan_columns_t<PrecX>(p, b0, b1, host_cols);
}

extern "C" int mgcu_plan_finish(mgcu_plan* p)
{
	MgcuContext* c = mgcu_ctx();
	cudaStream_t st = mgcu_stream();
	const int ng = std::max(p->d.ngates, 1);
	k_sum_parts<<<1, 32, 0, st>>>(p->part_f.as<double>(), p->grid_a, 2, p->out_f.as<double>());
	MGCU_LAUNCHED();
	if (p->d.want_grad || p->d.want_hess)
	{
		k_sum_parts<<<grid_cap(16L * ng, 128), 128, 0, st>>>(p->part_g.as<double>(), p->grid_a, 16L * ng, p->out_g.as<double>());
		MGCU_LAUNCHED();
		k_block_sum<<<(16 * p->d.nblocks + 127) / 128, 128, 0, st>>>(p->out_g.as<double>(), p->d_block.as<int>(), p->d.ngates, p->d.nblocks, p->out_blk.as<double>());
		MGCU_LAUNCHED();
	}
	if (p->d.want_hess)
	{
		const long mdim = 8L * p->d.nblocks;
		k_sum_parts<<<grid_cap(2 * mdim * mdim, 128), 128, 0, st>>>(p->part_h.as<double>(), p->grid_b, 2 * mdim * mdim, p->out_h.as<double>());
		MGCU_LAUNCHED();
		k_symm_diag<<<grid_cap(mdim * mdim, 256), 256, 0, st>>>(p->d.nblocks, p->out_h.as<double2>());
		MGCU_LAUNCHED();
		k_mirror<<<grid_cap(mdim * mdim, 256), 256, 0, st>>>(p->d.nblocks, p->out_h.as<double2>());
		MGCU_LAUNCHED();
	}
	return 0;
}

extern "C" int mgcu_plan_fetch(mgcu_plan* p, mgc* f, mgg* dblocks, mgc* hess)
{
	cudaStream_t st = mgcu_stream();
	if (f) MGCU_TRY(cudaMemcpyAsync(f, p->out_f.p, sizeof(double) * 2, cudaMemcpyDeviceToHost, st));
	if (dblocks && (p->d.want_grad || p->d.want_hess))
		MGCU_TRY(cudaMemcpyAsync(dblocks, p->out_blk.p, sizeof(double) * 16 * p->d.nblocks, cudaMemcpyDeviceToHost, st));
	if (hess && p->d.want_hess)
		MGCU_TRY(cudaMemcpyAsync(hess, p->out_h.p, sizeof(double) * 2 * 64 * (size_t)p->d.nblocks * p->d.nblocks, cudaMemcpyDeviceToHost, st));
	MGCU_TRY(cudaStreamSynchronize(st));
	return 0;
}

// projection of gradient and Hessian on the GPU (mgcu_algebra.cu)
extern int mgcu_project_dev(const mgg* vblocks_host, int nblocks, const double* dgrad_dev, const double* hess_dev,
	double* grad_vec, double* H);

extern "C" int mgcu_plan_project(mgcu_plan* p, const mgg* vblocks, double* grad_vec, double* H)
{
	return mgcu_project_dev(vblocks, p->d.nblocks, p->out_blk.as<double>(), p->d.want_hess ? p->out_h.as<double>() : nullptr, grad_vec, H);
}

extern "C" double mgcu_plan_time_ms(mgcu_plan* p, long b0, long b1, int steps, int flush_l2)
{
	MgcuContext* c = mgcu_ctx();
	if (flush_l2 && p->flush.alloc(512ull << 20)) return -1;
	p->ktime = true;
	p->kev_used = 0;
	struct Off { mgcu_plan* p; ~Off() { p->ktime = false; } } off{ p };
	double total = 0;
	for (int s = 0; s < steps; s++)
	{
		if (flush_l2 && cudaMemsetAsync(p->flush.p, s & 0xff, p->flush.n, mgcu_stream()) != cudaSuccess) return -1;
		cudaEventRecord(c->ev0, mgcu_stream());
		if (mgcu_plan_begin(p) || mgcu_plan_columns(p, b0, b1, nullptr) || mgcu_plan_finish(p)) return -1;
		cudaEventRecord(c->ev1, mgcu_stream());
		if (cudaEventSynchronize(c->ev1) != cudaSuccess) return -1;
		float ms = 0;
		cudaEventElapsedTime(&ms, c->ev0, c->ev1);
		total += ms;
	}
	return total;
}

// the target sweep the plan runs: cfg[0] kind (0 none: dense target or host map; 1 full; 2
// weight-restricted), cfg[1] tile bits, cfg[2] threads, cfg[3] live quartets per thread and
// iteration (weight-restricted) or columns per block (full)
extern "C" void mgcu_plan_target_config(const mgcu_plan* p, int* cfg)
{
	const bool circ = p->d.target && p->d.target->kind == 0;
	cfg[0] = circ ? (p->w_t ? 2 : 1) : 0;
	cfg[1] = p->kt_t;
	cfg[2] = p->threads_t;
	cfg[3] = p->w_t ? p->nq_t : p->nc_t;
}

// k_target launches of the last mgcu_plan_time_ms: their number and summed duration
extern "C" int mgcu_plan_target_kernel_ms(mgcu_plan* p, double* ms, long* launches)
{
	double t = 0;
	for (size_t i = 0; i + 1 < p->kev_used; i += 2)
	{
		float m = 0;
		MGCU_TRY(cudaEventElapsedTime(&m, p->kev[i], p->kev[i + 1]));
		t += m;
	}
	*ms = t;
	*launches = (long)(p->kev_used / 2);
	return 0;
}

// ======================================================================================
// Batches: many independent instances (brickwall fits against GPU circuit targets of
// any qubit count and depth), f and block gradients, in one persistent launch per phase
// and round; the launch sequence is captured once into a CUDA graph and replayed.
// ======================================================================================
namespace {

// fixed-order sums of one instance's item rows (one block per instance)
struct BatchRed
{
	const double* part_f;   // [nslots][2]
	const double* part_g;   // [nslots][ngates][16]
	const int* block;       // [ngates]
	double* out_f;          // [2]
	double* out_blk;        // [nblocks][16]
	int nslots, ngates, nblocks;
};

__global__ void k_batch_reduce(const BatchRed* __restrict__ rd)
{
	const BatchRed r = rd[blockIdx.x];
	if (threadIdx.x < 2)
	{
		double s = 0;
		for (int k = 0; k < r.nslots; k++) s += r.part_f[2 * k + threadIdx.x];
		r.out_f[threadIdx.x] = s;
	}
	for (int q = threadIdx.x; q < r.nblocks * 16; q += blockDim.x)
	{
		const int blk = q >> 4, e = q & 15;
		double s = 0;
		for (int g = 0; g < r.ngates; g++)
		{
			if (r.block[g] != blk) continue;
			for (int k = 0; k < r.nslots; k++) s += r.part_g[((size_t)k * r.ngates + g) * 16 + e];
		}
		r.out_blk[q] = s;
	}
}

struct BatchInst
{
	int L, nb, ngates, nblocks, kt_c, kt_t, nslots = 0, npass_t = 0;
	long S;
	Sched ws;
	std::vector<int> block;
	DevBuf d_pass, d_gate, d_mats, d_block, out_f, out_blk;
	TargetProg tp;                 // the batch's own copy of the target program
	mgcu_target* target;
	size_t smem_t, pm_off, smem_c;
	double col_cost;               // relative cost of one column
	bool big = false;              // enough columns to fill the GPU: its own kernels
	int grid_t = 0, grid_c = 0;    // standalone grids (big instances)
	long chunk = 0;                // columns per staged chunk (big instances)
	long part_off;                 // offsets (doubles) of part_f / part_g in the batch's partials
	long part_g_off;
};

} // namespace

struct mgcu_batch
{
	int prec, n, threads = 256;
	size_t tsize;
	std::unique_ptr<BatchInst[]> inst;
	DevBuf args_t, args_c, items, counters, scratch, parts, red;
	long slot_stride = 0, cache_stride = 0;
	size_t smem = 0;
	int grid[3] = { 0, 0, 0 }, nitems = 0;
	DevBuf stage, bsu, bsw, bcache;   // big instances: staged target columns, k_columns slots and caches
	std::vector<char> host_args;      // the instances' target and columns Args (kernel parameters of big ones)
	int class_beg[4] = { 0, 0, 0, 0 };   // items of tile classes 4, 8, any quartets per thread
	long graph_kernels = 0;        // kernel nodes per replay
	bool use_graph = true;         // false: plain launches (a batch run once)
	cudaGraph_t graph = nullptr;
	cudaGraphExec_t exec = nullptr;
	DevBuf flush;
	~mgcu_batch()
	{
		if (exec) cudaGraphExecDestroy(exec);
		if (graph) cudaGraphDestroy(graph);
	}
};

namespace {

template <class P>
static size_t target_smem(int kt, int threads, size_t tsize, size_t& pm_off)
{
	pm_off = ((size_t)1 << kt) * tsize + 2 * 128 * sizeof(unsigned) + std::max<size_t>((size_t)(threads / 32) * 16 * sizeof(double), 16 * 16);
	return pm_off + (size_t)MAXPM * 8 * tsize;
}

// Time the target sweep of t with tile bits kt on ncols columns (ms), using a temporary
// program and output buffer; used to choose each instance's tile size.
template <class P>
static double time_target(mgcu_target* t, int L, int kt, int threads, long ncols, int grid_cap)
{
	typedef typename P::T T;
	MgcuContext* c = mgcu_ctx();
	TargetProg tp;
	if (build_target_prog<P>(t, kt, threads, tp)) return -1;
	size_t pm_off;
	const size_t smem = target_smem<P>(kt, threads, sizeof(T), pm_off);
	DevBuf out;
	const long S = 1L << (L - 1);
	if (out.alloc(sizeof(T) * S * ncols)) return -1;
	Args<P> a;
	memset(&a, 0, sizeof(a));
	a.L = L; a.nb = L - 1; a.kt = kt; a.S = S;
	a.U.pass = tp.pass.as<PassRec>(); a.U.gate = tp.gate.as<GateRec>(); a.U.npass = (int)tp.sched.pass.size();
	a.utg = tp.tg.as<TGate>(); a.upm = tp.pm.as<int2>(); a.upmats = tp.pmats.as<T>(); a.pm_off = (unsigned)pm_off;
	a.b0 = 0; a.b1 = ncols; a.ucols = out.as<T>();
	int per_sm = 0;
	void (*kern)(Args<P>) = target_kernel<P>(kt, threads);
	if (!kern || cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, smem) != cudaSuccess || per_sm < 1) return -1;
	const int grid = (int)std::min<long>(std::min<long>((long)c->nsm * per_sm, grid_cap), ncols);
	double best = -1;
	for (int rep = 0; rep < 2; rep++)
	{
		cudaEventRecord(c->ev0, mgcu_stream());
		kern<<<grid, threads, smem, mgcu_stream()>>>(a);
		cudaEventRecord(c->ev1, mgcu_stream());
		if (cudaEventSynchronize(c->ev1) != cudaSuccess) return -1;
		float ms = 0;
		cudaEventElapsedTime(&ms, c->ev0, c->ev1);
		if (rep == 1) best = ms;   // the first run warms caches and code
	}
	return best;
}

template <class P>
static int batch_build(mgcu_batch* B, const mgcu_batch_inst* d, int tune)
{
	typedef typename P::T T;
	MgcuContext* c = mgcu_ctx();
	const int threads = B->threads;
	{
		const int e = set_smem_attr<P>();
		if (e) return e;
	}
	const int kt_default = sizeof(T) >= 16 ? 12 : 13;
	// tile choice per distinct (target, L): time the candidates on a column sample
	std::map<std::pair<mgcu_target*, int>, int> tuned;
	for (int i = 0; i < B->n; i++)
	{
		BatchInst& I = B->inst[i];
		const mgcu_batch_inst& D = d[i];
		I.L = D.L; I.nb = D.L - 1; I.S = 1L << (D.L - 1); I.ngates = D.ngates; I.nblocks = D.nblocks; I.target = D.target;
		I.block.assign(D.block, D.block + D.ngates);
		I.kt_c = std::min(kt_default, I.nb);
		const std::pair<mgcu_target*, int> key(D.target, D.L);
		auto it = tuned.find(key);
		if (it == tuned.end() && tune && D.target->tuned_kt[P::kId][D.L] > 0)
			it = tuned.emplace(key, D.target->tuned_kt[P::kId][D.L]).first;
		if (it == tuned.end())
		{
			int best_kt = std::min(kt_default, I.nb);
			if (tune && I.nb > 10)
			{
				double best_ms = -1;
				const long ncols = std::min<long>(1L << D.L, (long)c->nsm * 4);
				for (int kt = 10; kt <= std::min(kt_default, I.nb); kt++)
				{
					const double ms = time_target<P>(D.target, D.L, kt, threads, ncols, c->nsm * 2);
					if (ms > 0 && (best_ms < 0 || ms < best_ms)) { best_ms = ms; best_kt = kt; }
				}
			}
			it = tuned.emplace(key, best_kt).first;
			if (tune) D.target->tuned_kt[P::kId][D.L] = best_kt;
		}
		I.kt_t = it->second;
		int e = build_target_prog<P>(D.target, I.kt_t, threads, I.tp);
		if (e) return e;
		I.npass_t = (int)I.tp.sched.pass.size();
		I.smem_t = target_smem<P>(I.kt_t, threads, sizeof(T), I.pm_off);
		I.smem_c = ((size_t)1 << I.kt_c) * sizeof(T) + 2 * 128 * sizeof(unsigned) + red_bytes(threads);
		schedule(I.L, I.kt_c, D.wires, D.ngates, false, I.ws);
		e = upload_sched(I.ws, I.d_pass, I.d_gate);
		if (!e) e = I.d_mats.alloc(sizeof(T) * 8 * std::max(D.ngates, 1));
		if (!e) e = I.d_block.alloc(sizeof(int) * std::max(D.ngates, 1));
		if (!e) e = I.out_f.alloc(sizeof(double) * 2);
		if (!e) e = I.out_blk.alloc(sizeof(double) * 16 * std::max(D.nblocks, 1));
		if (e) return e;
		MGCU_TRY(cudaMemcpy(I.d_block.p, D.block, sizeof(int) * D.ngates, cudaMemcpyHostToDevice));
		I.col_cost = (double)I.S * ((double)mgcu_target_sweep_gates(D.target) + 3.0 * D.ngates);
		B->smem = std::max(B->smem, std::max(I.smem_t, I.smem_c));
		B->slot_stride = std::max(B->slot_stride, I.S);
		if (D.want_grad) B->cache_stride = std::max(B->cache_stride, I.S * D.ngates);
	}
	// one batched kernel per tile class; each also holds one static shared int: ask for
	// exactly what it uses
	void (*const kb[3])(const Args<P>*, const Args<P>*, const BatchItem*, int, int*, T*, long, long) = { k_batch<P, 4>, k_batch<P, 8>, k_batch<P, 0> };
	for (int k = 0; k < 3; k++)
	{
		MGCU_TRY(cudaFuncSetAttribute(kb[k], cudaFuncAttributeMaxDynamicSharedMemorySize, (int)B->smem));
		int pb = 0;
		MGCU_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&pb, kb[k], threads, B->smem));
		if (pb < 1) { mg_set_error("batch: a block does not fit on an SM"); return MG_ERR_ARG; }
		B->grid[k] = c->nsm * pb;
	}
	auto tile_class = [&](const BatchInst& I) {
		const long Q = 1L << (I.kt_t - 2);
		return (Q == 4L * threads) ? 0 : (Q == 8L * threads) ? 1 : 2;
	};

	// Instances with at least four columns per resident block run the two standalone
	// kernels (k_target into a staged chunk, then k_columns), which are faster per column
	// than the fused kernel; the others share the fused persistent launch.
	size_t stage_bytes = 0, slot_max = 0, cache_max = 0;
	int grid_c_max = 0;
	for (int i = 0; i < B->n; i++)
	{
		BatchInst& I = B->inst[i];
		void (*kt_)(Args<P>) = target_kernel<P>(I.kt_t, threads);
		int pt = 0, pc = 0;
		MGCU_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&pt, kt_, threads, I.smem_t));
		MGCU_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&pc, k_columns<P, false>, threads, I.smem_c));
		I.grid_t = c->nsm * std::max(pt, 1);
		I.grid_c = c->nsm * std::max(pc, 1);
		I.big = (1L << I.L) >= 4L * std::max(I.grid_t, I.grid_c);
		if (!I.big) continue;
		I.chunk = std::max(1L, std::min(1L << I.L, (long)((8ull << 30) / ((size_t)I.S * sizeof(T)))));
		stage_bytes = std::max(stage_bytes, sizeof(T) * (size_t)I.S * (size_t)I.chunk);
		slot_max = std::max(slot_max, (size_t)I.S);
		if (d[i].want_grad) cache_max = std::max(cache_max, (size_t)I.S * (size_t)I.ngates);
		grid_c_max = std::max(grid_c_max, I.grid_c);
	}
	if (stage_bytes)
	{
		int e = B->stage.alloc(stage_bytes);
		if (!e) e = B->bsu.alloc(sizeof(T) * slot_max * grid_c_max);
		if (!e) e = B->bsw.alloc(sizeof(T) * slot_max * grid_c_max);
		if (!e && cache_max) e = B->bcache.alloc(sizeof(T) * cache_max * grid_c_max);
		if (e) return e;
	}

	// work items of the other instances: about 16 per block, never more than an
	// instance's columns, largest first
	double total = 0;
	for (int i = 0; i < B->n; i++) if (!B->inst[i].big) total += B->inst[i].col_cost * (double)(1L << B->inst[i].L);
	const double item_cost = total / (16.0 * B->grid[0]);
	struct HostItem { BatchItem it; double cost; };
	std::vector<HostItem> all;
	for (int i = 0; i < B->n; i++)
	{
		BatchInst& I = B->inst[i];
		if (I.big) { I.nslots = I.grid_c; continue; }   // partial rows: one per k_columns block
		const long N = 1L << I.L;
		const long per = std::max(1L, std::min(N, (long)(item_cost / I.col_cost)));
		for (long b0 = 0; b0 < N; b0 += per)
		{
			HostItem h;
			h.it.inst = i; h.it.slot = I.nslots++; h.it.b0 = b0; h.it.b1 = std::min(N, b0 + per);
			h.cost = I.col_cost * (double)(h.it.b1 - h.it.b0);
			all.push_back(h);
		}
	}
	// by tile class, then largest first
	std::vector<int> cls(B->n);
	for (int i = 0; i < B->n; i++) cls[i] = tile_class(B->inst[i]);
	std::stable_sort(all.begin(), all.end(), [&](const HostItem& x, const HostItem& y) {
		const int cx = cls[x.it.inst], cy = cls[y.it.inst];
		return cx != cy ? cx < cy : x.cost > y.cost;
	});
	for (int k = 0; k <= 3; k++) B->class_beg[k] = 0;
	{
		int n = 0;
		for (int k = 0; k < 3; k++)
		{
			B->class_beg[k] = n;
			for (const HostItem& h : all) if (cls[h.it.inst] == k) n++;
		}
		B->class_beg[3] = n;
	}
	std::vector<BatchItem> items;
	for (const HostItem& h : all) items.push_back(h.it);
	B->nitems = (int)items.size();

	// partial rows of every instance in one buffer
	long off = 0;
	for (int i = 0; i < B->n; i++)
	{
		BatchInst& I = B->inst[i];
		I.part_off = off; off += 2L * I.nslots;
		I.part_g_off = off; off += 16L * I.nslots * std::max(I.ngates, 1);
	}
	int e = B->parts.alloc(sizeof(double) * std::max(off, 1L));
	const int gmax = std::max(B->grid[0], std::max(B->grid[1], B->grid[2]));
	if (!e) e = B->scratch.alloc(sizeof(T) * (size_t)gmax * (size_t)(3 * B->slot_stride + B->cache_stride));
	if (!e) e = B->items.alloc(sizeof(BatchItem) * std::max<size_t>(items.size(), 1));
	if (!e) e = B->counters.alloc(sizeof(int) * 4);
	if (!e) e = B->args_t.alloc(sizeof(Args<P>) * B->n);
	if (!e) e = B->args_c.alloc(sizeof(Args<P>) * B->n);
	if (!e) e = B->red.alloc(sizeof(BatchRed) * B->n);
	if (e) return e;
	MGCU_TRY(cudaMemcpy(B->items.p, items.data(), sizeof(BatchItem) * items.size(), cudaMemcpyHostToDevice));
	std::vector<Args<P>> at(B->n), ac(B->n);
	std::vector<BatchRed> rd(B->n);
	double* parts = B->parts.as<double>();
	for (int i = 0; i < B->n; i++)
	{
		BatchInst& I = B->inst[i];
		Args<P>& a = at[i];
		memset(&a, 0, sizeof(a));
		a.L = I.L; a.nb = I.nb; a.kt = I.kt_t; a.S = I.S;
		a.U.pass = I.tp.pass.as<PassRec>(); a.U.gate = I.tp.gate.as<GateRec>(); a.U.npass = (int)I.tp.sched.pass.size();
		a.utg = I.tp.tg.as<TGate>(); a.upm = I.tp.pm.as<int2>(); a.upmats = I.tp.pmats.as<T>(); a.pm_off = (unsigned)I.pm_off;
		Args<P>& w = ac[i];
		memset(&w, 0, sizeof(w));
		w.L = I.L; w.nb = I.nb; w.kt = I.kt_c; w.S = I.S;
		w.W.pass = I.d_pass.as<PassRec>(); w.W.gate = I.d_gate.as<GateRec>(); w.W.npass = (int)I.ws.pass.size();
		w.wm = I.d_mats.as<T>(); w.ngates = I.ngates; w.want_grad = d[i].want_grad ? 1 : 0;
		w.part_f = parts + I.part_off; w.part_g = parts + I.part_g_off;
		BatchRed& r = rd[i];
		r.part_f = parts + I.part_off; r.part_g = parts + I.part_g_off; r.block = I.d_block.as<int>();
		r.out_f = I.out_f.as<double>(); r.out_blk = I.out_blk.as<double>();
		r.nslots = I.nslots; r.ngates = I.ngates; r.nblocks = I.nblocks;
	}
	MGCU_TRY(cudaMemcpy(B->args_t.p, at.data(), sizeof(Args<P>) * B->n, cudaMemcpyHostToDevice));
	MGCU_TRY(cudaMemcpy(B->args_c.p, ac.data(), sizeof(Args<P>) * B->n, cudaMemcpyHostToDevice));
	B->host_args.resize(sizeof(Args<P>) * 2 * B->n);
	memcpy(B->host_args.data(), at.data(), sizeof(Args<P>) * B->n);
	memcpy(B->host_args.data() + sizeof(Args<P>) * B->n, ac.data(), sizeof(Args<P>) * B->n);
	MGCU_TRY(cudaMemcpy(B->red.p, rd.data(), sizeof(BatchRed) * B->n, cudaMemcpyHostToDevice));
	return 0;
}

// the launch sequence of one batch evaluation on the library's stream
template <class P>
static int batch_issue(mgcu_batch* B)
{
	typedef typename P::T T;
	cudaStream_t st = mgcu_stream();
	MGCU_TRY(cudaMemsetAsync(B->parts.p, 0, B->parts.n, st));
	MGCU_TRY(cudaMemsetAsync(B->counters.p, 0, B->counters.n, st));
	const Args<P>* hat = reinterpret_cast<const Args<P>*>(B->host_args.data());
	const Args<P>* hac = hat + B->n;
	for (int i = 0; i < B->n; i++)
	{
		const BatchInst& I = B->inst[i];
		if (!I.big) continue;
		void (*kt_)(Args<P>) = target_kernel<P>(I.kt_t, B->threads);
		const long N = 1L << I.L;
		for (long c0 = 0; c0 < N; c0 += I.chunk)
		{
			const long c1 = std::min(N, c0 + I.chunk);
			Args<P> a = hat[i];
			a.b0 = c0; a.b1 = c1; a.ucols = B->stage.as<T>();
			kt_<<<(int)std::min<long>(I.grid_t, c1 - c0), B->threads, I.smem_t, st>>>(a);
			MGCU_LAUNCHED();
			Args<P> w = hac[i];
			w.b0 = c0; w.b1 = c1; w.dense = B->stage.as<T>(); w.dense_b0 = c0;
			w.su = B->bsu.as<T>(); w.sw = B->bsw.as<T>();
			w.cache = w.want_grad ? B->bcache.as<T>() : nullptr;
			k_columns<P, false><<<(int)std::min<long>(I.grid_c, c1 - c0), B->threads, I.smem_c, st>>>(w);
			MGCU_LAUNCHED();
		}
	}
	void (*const kb[3])(const Args<P>*, const Args<P>*, const BatchItem*, int, int*, T*, long, long) = { k_batch<P, 4>, k_batch<P, 8>, k_batch<P, 0> };
	for (int k = 0; k < 3; k++)
	{
		const int i0 = B->class_beg[k], ni = B->class_beg[k + 1] - i0;
		if (ni == 0) continue;
		kb[k]<<<std::min(B->grid[k], ni), B->threads, B->smem, st>>>(B->args_t.as<Args<P>>(), B->args_c.as<Args<P>>(),
			B->items.as<BatchItem>() + i0, ni, B->counters.as<int>() + k, B->scratch.as<T>(), B->slot_stride, B->cache_stride);
		MGCU_LAUNCHED();
	}
	k_batch_reduce<<<B->n, 128, 0, st>>>(B->red.as<BatchRed>());
	MGCU_LAUNCHED();
	return 0;
}

template <class P>
static int batch_issue_graph(mgcu_batch* B)
{
	cudaStream_t st = mgcu_stream();
	if (!B->use_graph) return batch_issue<P>(B);
	if (!B->exec)
	{
		MGCU_TRY(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
		const long n0 = mgcu_launch_count();
		const int e = batch_issue<P>(B);
		B->graph_kernels = mgcu_launch_count() - n0;
		mgcu_count_launch(-B->graph_kernels);   // counted when the graph runs
		cudaGraph_t g = nullptr;
		const cudaError_t ce = cudaStreamEndCapture(st, &g);
		if (e || ce != cudaSuccess) { if (g) cudaGraphDestroy(g); if (!e) MGCU_TRY(ce); return e ? e : MG_ERR_DEVICE; }
		B->graph = g;
		MGCU_TRY(cudaGraphInstantiate(&B->exec, B->graph, 0));
	}
	MGCU_TRY(cudaGraphLaunch(B->exec, st));
	mgcu_count_launch(B->graph_kernels);
	return 0;
}

} // namespace

extern "C" mgcu_batch* mgcu_batch_create(int n, const mgcu_batch_inst* d, int precision, int tune, int use_graph)
{
	if (!mgcu_ctx()) return nullptr;
	if (n < 1) { mg_set_error("a batch needs at least one instance"); return nullptr; }
	for (int i = 0; i < n; i++)
		if (!d[i].target || d[i].target->kind != 0 || d[i].target->L != d[i].L || d[i].L < 4 || d[i].L > 30 || d[i].ngates < 1)
		{
			mg_set_error("batch instance %d: needs a GPU circuit target on its qubits (4..30) and at least one gate", i);
			return nullptr;
		}
	mgcu_batch* B = new mgcu_batch();
	B->prec = precision; B->n = n; B->tsize = prec_tsize(precision); B->use_graph = use_graph != 0;
	B->inst.reset(new BatchInst[n]);
	int e;
	if (precision == MG_PREC_FP64_ID) e = batch_build<PrecD>(B, d, tune);
	else if (precision == MG_PREC_FP32_ID) e = batch_build<PrecF>(B, d, tune);
	else e = batch_build<PrecX>(B, d, tune);
	if (e) { delete B; return nullptr; }
	return B;
}

extern "C" void mgcu_batch_destroy(mgcu_batch* B) { delete B; }

extern "C" int mgcu_batch_set_gates(mgcu_batch* B, int i, const mgg* gates)
{
	if (i < 0 || i >= B->n) { mg_set_error("batch instance %d out of range", i); return MG_ERR_ARG; }
	BatchInst& I = B->inst[i];
	if (B->prec == MG_PREC_FP64_ID) return upload_mats<PrecD>(gates, I.ngates, I.d_mats);
	if (B->prec == MG_PREC_FP32_ID) return upload_mats<PrecF>(gates, I.ngates, I.d_mats);
	return upload_mats<PrecX>(gates, I.ngates, I.d_mats);
}

// one evaluation of every instance (graph replay; the first call captures the graph)
// the batch's work queued on the calling thread's stream, without waiting for it
extern "C" int mgcu_batch_issue(mgcu_batch* B)
{
	if (B->prec == MG_PREC_FP64_ID) return batch_issue_graph<PrecD>(B);
	if (B->prec == MG_PREC_FP32_ID) return batch_issue_graph<PrecF>(B);
	return batch_issue_graph<PrecX>(B);
}

extern "C" int mgcu_batch_run(mgcu_batch* B)
{
	const int e = mgcu_batch_issue(B);
	if (e) return e;
	MGCU_TRY(cudaStreamSynchronize(mgcu_stream()));
	return 0;
}

extern "C" int mgcu_batch_fetch(mgcu_batch* B, int i, mgc* f, mgg* dblocks)
{
	if (i < 0 || i >= B->n) { mg_set_error("batch instance %d out of range", i); return MG_ERR_ARG; }
	BatchInst& I = B->inst[i];
	if (f) MGCU_TRY(cudaMemcpy(f, I.out_f.p, sizeof(double) * 2, cudaMemcpyDeviceToHost));
	if (dblocks) MGCU_TRY(cudaMemcpy(dblocks, I.out_blk.p, sizeof(double) * 16 * I.nblocks, cudaMemcpyDeviceToHost));
	return 0;
}

extern "C" int mgcu_batch_project(mgcu_batch* B, int i, const mgg* vblocks, double* grad_vec)
{
	if (i < 0 || i >= B->n) { mg_set_error("batch instance %d out of range", i); return MG_ERR_ARG; }
	BatchInst& I = B->inst[i];
	return mgcu_project_dev(vblocks, I.nblocks, I.out_blk.as<double>(), nullptr, grad_vec, nullptr);
}

extern "C" int mgcu_batch_info(const mgcu_batch* B, int i, int* target_tile_bits, int* target_passes, int* items)
{
	if (i < 0 || i >= B->n) { mg_set_error("batch instance %d out of range", i); return MG_ERR_ARG; }
	const BatchInst& I = B->inst[i];
	if (target_tile_bits) *target_tile_bits = I.kt_t;
	if (target_passes) *target_passes = I.npass_t;
	if (items) *items = I.nslots;
	return 0;
}

extern "C" double mgcu_batch_time_ms(mgcu_batch* B, int steps, int flush_l2)
{
	MgcuContext* c = mgcu_ctx();
	if (flush_l2 && B->flush.alloc(512ull << 20)) return -1;
	double total = 0;
	for (int s = 0; s < steps; s++)
	{
		if (flush_l2 && cudaMemsetAsync(B->flush.p, s & 0xff, B->flush.n, mgcu_stream()) != cudaSuccess) return -1;
		cudaEventRecord(c->ev0, mgcu_stream());
		int e;
		if (B->prec == MG_PREC_FP64_ID) e = batch_issue_graph<PrecD>(B);
		else if (B->prec == MG_PREC_FP32_ID) e = batch_issue_graph<PrecF>(B);
		else e = batch_issue_graph<PrecX>(B);
		if (e) return -1;
		cudaEventRecord(c->ev1, mgcu_stream());
		if (cudaEventSynchronize(c->ev1) != cudaSuccess) return -1;
		float ms = 0;
		cudaEventElapsedTime(&ms, c->ev0, c->ev1);
		total += ms;
	}
	return total;
}

// ======================================================================================
// Allocation-free evaluation: f and layer gradients of a brickwall against a target
// circuit, with every workspace in one fixed device array instead of cudaMalloc'd
// buffers.  For callers that must not allocate GPU memory mid-run (see mg_gb300.h).
// ======================================================================================
namespace {

constexpr int NA_MAX_QUBITS = 10;          // one shared-memory tile holds a whole sector
constexpr int NA_MAX_FIT_GATES = 64;       // nlayers * nqubits / 2
constexpr int NA_MAX_TARGET_GATES = 4096;
constexpr int NA_BLOCKS = 64;              // resident columns at a time
constexpr size_t NA_S = (size_t)1 << (NA_MAX_QUBITS - 1);

// byte offsets inside the scratch array (every region 256-byte aligned)
constexpr size_t na_al(size_t x) { return (x + 255) / 256 * 256; }
constexpr size_t NA_SU = 0;
constexpr size_t NA_SW = NA_SU + na_al(sizeof(double2) * NA_BLOCKS * NA_S);
constexpr size_t NA_CACHE = NA_SW + na_al(sizeof(double2) * NA_BLOCKS * NA_S);
constexpr size_t NA_PART_F = NA_CACHE + na_al(sizeof(double2) * NA_BLOCKS * NA_MAX_FIT_GATES * NA_S);
constexpr size_t NA_PART_G = NA_PART_F + na_al(sizeof(double) * 2 * NA_BLOCKS);
constexpr size_t NA_OUT_F = NA_PART_G + na_al(sizeof(double) * 16 * NA_MAX_FIT_GATES * NA_BLOCKS);
constexpr size_t NA_OUT_G = NA_OUT_F + na_al(sizeof(double) * 2);
constexpr size_t NA_OUT_BLK = NA_OUT_G + na_al(sizeof(double) * 16 * NA_MAX_FIT_GATES);
constexpr size_t NA_WMAT = NA_OUT_BLK + na_al(sizeof(double) * 16 * NA_MAX_FIT_GATES);
constexpr size_t NA_UMAT = NA_WMAT + na_al(sizeof(double2) * 8 * NA_MAX_FIT_GATES);
constexpr size_t NA_PASS = NA_UMAT + na_al(sizeof(double2) * 8 * NA_MAX_TARGET_GATES);
constexpr size_t NA_GATE = NA_PASS + na_al(sizeof(PassRec) * 2);
constexpr size_t NA_BLOCK = NA_GATE + na_al(sizeof(GateRec) * (NA_MAX_FIT_GATES + NA_MAX_TARGET_GATES));
constexpr size_t NA_BYTES = NA_BLOCK + na_al(sizeof(int) * NA_MAX_FIT_GATES);

// host staging for the small inputs: static storage, no heap
PassRec na_pass_h[2];
GateRec na_gate_h[NA_MAX_FIT_GATES + NA_MAX_TARGET_GATES];
double2 na_wmat_h[8 * NA_MAX_FIT_GATES];
double2 na_umat_h[8 * NA_MAX_TARGET_GATES];
int na_block_h[NA_MAX_FIT_GATES];
int na_wires_h[2 * NA_MAX_FIT_GATES];
double na_out_h[2 + 16 * NA_MAX_FIT_GATES];
unsigned char* na_base[64];                // scratch address per device, set at first use

// one pass with every compact bit local (the sector fits one tile)
void na_single_pass(int L, const int* wires, int ng, int gofs, PassRec& pr, GateRec* recs)
{
	const int nb = L - 1;
	memset(&pr, 0, sizeof(pr));
	for (int b = 0; b < nb; b++) pr.lbits[b] = b;
	pr.nnl = 0;
	pr.gbeg = gofs;
	pr.gend = gofs + ng;
	for (int g = 0; g < ng; g++)
	{
		GateRec r;
		const int a = compact_bit(L, wires[2 * g]), b = compact_bit(L, wires[2 * g + 1]);
		r.g = g;
		r.type = (a >= 0 && b >= 0) ? 0 : (b < 0 ? 1 : 2);
		r.la = a;
		r.lb = b;
		const int used = r.type == 1 ? r.la : r.lb;
		r.lc = (used == 0) ? 1 : 0;
		recs[gofs + g] = r;
	}
}

}  // namespace

// Every GPU that loads this library reserves this array until the process exits.
static __device__ __align__(256) unsigned char g_noalloc_scratch[NA_BYTES];

// C linkage: the types of mg_gb300.h's declaration (struct matchgate, numeric) share these layouts
extern "C" int mg_noalloc_brickwall_target_and_gradient(const void* ugates, int ungates, const int uwires[],
	const void* vlist, int nlayers, int nqubits, const int* perms[], double* fval, void* dvlist)
{
	const int L = nqubits, half = L / 2, ng = nlayers * half;
	if (L < 4 || L > NA_MAX_QUBITS || L % 2 || nlayers < 1 || ng > NA_MAX_FIT_GATES || ungates < 0 || ungates > NA_MAX_TARGET_GATES)
	{
		mg_set_error("mg_noalloc_brickwall_target_and_gradient: sizes outside its fixed workspace (need even 4 <= nqubits <= %d, "
			"nlayers*nqubits/2 <= %d, target gates <= %d; got nqubits=%d nlayers=%d target gates=%d)",
			NA_MAX_QUBITS, NA_MAX_FIT_GATES, NA_MAX_TARGET_GATES, L, nlayers, ungates);
		return MG_ERR_ARG;
	}
	for (int g = 0; g < 2 * ungates; g++)
		if (uwires[g] < 0 || uwires[g] >= L || (g % 2 && uwires[g] == uwires[g - 1]))
		{
			mg_set_error("mg_noalloc_brickwall_target_and_gradient: invalid wires of target gate %d", g / 2);
			return MG_ERR_ARG;
		}
	// each layer's wiring must be a permutation: a gate whose two wires coincide has no
	// quartet layout (the regular plans reject it the same way)
	for (int i = 0; i < nlayers; i++)
	{
		unsigned seen = 0;
		for (int p = 0; p < L; p++)
		{
			const int q = perms[i][p];
			if (q < 0 || q >= L || (seen >> q) & 1u)
			{
				mg_set_error("mg_noalloc_brickwall_target_and_gradient: invalid permutation of layer %d "
					"(wire %d out of range or repeated)", i, q);
				return MG_ERR_ARG;
			}
			seen |= 1u << q;
		}
	}
	mgcu_lock();
	MgcuContext* c = mgcu_ctx();
	if (!c) { mgcu_unlock(); return MG_ERR_DEVICE; }
	int rc = 0;
	// set-up once per device, with that device current: the device address of the array
	if (!na_base[c->device])
	{
		void* p = nullptr;
		cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
		if (e != cudaSuccess) { rc = mgcu_check(e, "cudaGetSymbolAddress", __FILE__, __LINE__); mgcu_unlock(); return rc; }
		na_base[c->device] = (unsigned char*)p;
	}
	unsigned char* base = na_base[c->device];
	const mgg* W = reinterpret_cast<const mgg*>(vlist);
	const mgg* U = reinterpret_cast<const mgg*>(ugates);
	for (int i = 0; i < nlayers; i++)
		for (int p = 0; p < half; p++)
		{
			const int g = i * half + p;
			na_wires_h[2 * g] = perms[i][2 * p];
			na_wires_h[2 * g + 1] = perms[i][2 * p + 1];
			na_block_h[g] = i;
			for (int q = 0; q < 4; q++)
			{
				na_wmat_h[8 * g + q] = make_double2(W[i].c[q].re, W[i].c[q].im);
				na_wmat_h[8 * g + 4 + q] = make_double2(W[i].k[q].re, W[i].k[q].im);
			}
		}
	for (int g = 0; g < ungates; g++)
		for (int q = 0; q < 4; q++)
		{
			na_umat_h[8 * g + q] = make_double2(U[g].c[q].re, U[g].c[q].im);
			na_umat_h[8 * g + 4 + q] = make_double2(U[g].k[q].re, U[g].k[q].im);
		}
	na_single_pass(L, na_wires_h, ng, 0, na_pass_h[0], na_gate_h);
	na_single_pass(L, uwires, ungates, ng, na_pass_h[1], na_gate_h);
	cudaStream_t st = mgcu_stream();
	const long ncols = 1L << L;
	const int grid = (int)std::min<long>(NA_BLOCKS, ncols);
	const int kt = L - 1;
	const int threads = std::max(32, std::min(256, 1 << (kt - 2)));
	const size_t smem = ((size_t)1 << kt) * sizeof(double2) + 2 * 128 * sizeof(unsigned) + red_bytes(threads);
#define NA_TRY(x) do { cudaError_t _e = (x); if (_e != cudaSuccess) { rc = mgcu_check(_e, #x, __FILE__, __LINE__); goto done; } } while (0)
	NA_TRY(cudaMemcpyAsync(base + NA_WMAT, na_wmat_h, sizeof(double2) * 8 * ng, cudaMemcpyHostToDevice, st));
	if (ungates) NA_TRY(cudaMemcpyAsync(base + NA_UMAT, na_umat_h, sizeof(double2) * 8 * ungates, cudaMemcpyHostToDevice, st));
	NA_TRY(cudaMemcpyAsync(base + NA_PASS, na_pass_h, sizeof(PassRec) * 2, cudaMemcpyHostToDevice, st));
	NA_TRY(cudaMemcpyAsync(base + NA_GATE, na_gate_h, sizeof(GateRec) * (ng + ungates), cudaMemcpyHostToDevice, st));
	NA_TRY(cudaMemcpyAsync(base + NA_BLOCK, na_block_h, sizeof(int) * ng, cudaMemcpyHostToDevice, st));
	// the partial sums accumulate: clear them (the array keeps the previous call's contents)
	NA_TRY(cudaMemsetAsync(base + NA_PART_F, 0, sizeof(double) * 2 * NA_BLOCKS, st));
	NA_TRY(cudaMemsetAsync(base + NA_PART_G, 0, sizeof(double) * 16 * ng * NA_BLOCKS, st));
	{
		Args<PrecD> a;
		memset(&a, 0, sizeof(a));
		a.L = L; a.nb = L - 1; a.kt = kt; a.S = ncols >> 1;
		a.W.pass = reinterpret_cast<const PassRec*>(base + NA_PASS);
		a.W.gate = reinterpret_cast<const GateRec*>(base + NA_GATE);
		a.W.npass = 1;
		a.U.pass = reinterpret_cast<const PassRec*>(base + NA_PASS) + 1;
		a.U.gate = reinterpret_cast<const GateRec*>(base + NA_GATE);
		a.U.npass = 1;
		a.wm = reinterpret_cast<const double2*>(base + NA_WMAT);
		a.um = reinterpret_cast<const double2*>(base + NA_UMAT);
		a.ngates = ng;
		a.b0 = 0; a.b1 = ncols;
		a.su = reinterpret_cast<double2*>(base + NA_SU);
		a.sw = reinterpret_cast<double2*>(base + NA_SW);
		a.cache = reinterpret_cast<double2*>(base + NA_CACHE);
		a.want_grad = 1;
		a.part_f = reinterpret_cast<double*>(base + NA_PART_F);
		a.part_g = reinterpret_cast<double*>(base + NA_PART_G);
		k_columns<PrecD, true><<<grid, threads, smem, st>>>(a);
		mgcu_count_launch();
		NA_TRY(cudaGetLastError());
		k_sum_parts<<<1, 32, 0, st>>>(a.part_f, grid, 2, reinterpret_cast<double*>(base + NA_OUT_F));
		mgcu_count_launch();
		k_sum_parts<<<grid_cap(16L * ng, 128), 128, 0, st>>>(a.part_g, grid, 16L * ng, reinterpret_cast<double*>(base + NA_OUT_G));
		mgcu_count_launch();
		k_block_sum<<<(16 * nlayers + 127) / 128, 128, 0, st>>>(reinterpret_cast<double*>(base + NA_OUT_G), reinterpret_cast<const int*>(base + NA_BLOCK),
			ng, nlayers, reinterpret_cast<double*>(base + NA_OUT_BLK));
		mgcu_count_launch();
		NA_TRY(cudaGetLastError());
	}
	NA_TRY(cudaMemcpyAsync(na_out_h, base + NA_OUT_F, sizeof(double) * 2, cudaMemcpyDeviceToHost, st));
	NA_TRY(cudaMemcpyAsync(na_out_h + 2, base + NA_OUT_BLK, sizeof(double) * 16 * nlayers, cudaMemcpyDeviceToHost, st));
	NA_TRY(cudaStreamSynchronize(st));
	fval[0] = na_out_h[0];
	fval[1] = na_out_h[1];
	memcpy(dvlist, na_out_h + 2, sizeof(double) * 16 * nlayers);
done:
#undef NA_TRY
	mgcu_unlock();
	return rc;
}
