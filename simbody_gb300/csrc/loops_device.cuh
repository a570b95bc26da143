// loops_device.cuh -- Constraint::Ball loop closures on the FP64 chain
// driver: the multipliers of the loop forward dynamics and the integrator's
// position and velocity projections. Textually included by abi_device.cuh
// inside namespace sbg (it uses that file's records, kinematics and sweeps).
//
// Constraint::Ball (ConstraintImpl.h:1835-1993) keeps station P (station 1
// on body 1) and S (station 2 on body 2) together: perr = p_S - p_P. The
// velocity and acceleration errors and the constraint forces use C, the
// material point of body 1 coincident with S:
//   verr = v_S - v_C,  aerr = a_S - a_C,  +lambda at S on body 2, -lambda at C.
// G = d verr / du is never formed: G^T x is the mobility force of point
// forces x at S and -x at C (an inward sweep), G v the point-velocity
// difference after an outward sweep.
//
// Loop forward dynamics (SimbodyMatterSubsystemRep.cpp:5076-5152, 3512-3558):
// with the tree solution udot_t,  (G M^-1 G^T) lambda = aerr(udot_t),
// udot = udot_t - M^-1 G^T lambda. Column j of G M^-1 G^T is the point
// acceleration difference of an M^-1 sweep driven by unit forces of
// equation j. The m x m system (m <= 12) is factored in FP64 by a Cholesky
// with symmetric pivoting that drops the equations a redundant closure
// repeats (loopCholFactor); the reference's rank-revealing QTZ gives the same
// constraint forces.
//
// Projections (SimbodyMatterSubsystemRep.cpp:4096-4442 and 4664-4943):
//   position  du = D G^T (G D G^T)^-1 perr, q -= N(q) du, full Newton until
//             RMS(perr) <= 0.1 tol (at most 20 iterations), D = 4|q|^2 on the
//             rotational mobilities of quaternion joints and 1 elsewhere
//             (the weighting of the reference's (P N^+) minimum-norm solve,
//             Rotation.h:742-748), then quaternions are normalized;
//   velocity  du = E^2 G^T (G E^2 G^T)^-1 verr, E = max(|u|, 1) at entry,
//             one factorization, at most 7 iterations.
// With localOnly a growing norm stops the iteration and undoes the last
// step; a result worse than the entry state is restored.
//
// Unit constraint forces act on the loop bodies only, so the inward half of
// every sweep is zero away from the loop bodies' paths to Ground (rows with
// F_LOOPPATH), and the slot values the Gram columns, perr and verr need lie
// on those paths: the sweeps, the kinematics of the projections and the
// accumulator clears visit path rows only. The one sweep whose outward half
// reaches every body (the constraint-force correction of udot) takes zero
// eps off the path. Skipped rows would have contributed exact zeros, so the
// results are the same as full sweeps.

// Loop-closure records through either driver's layout: element f of record
// rec at rec * a + f * b, with (a, b) = (s, s) for the interleaved tiles of
// the one-thread driver (stride s) and (W, 1) for the record-major rows of
// the level-parallel driver (record width W; the bodies, then the slot
// records).
template <class R> struct ScrGenT {
    R* p;
    int a, b;
    __device__ __forceinline__ R& operator()(int rec, int f) const { return p[rec * a + f * b]; }
};
using ScrGen = ScrGenT<double>;
using SC64 = ScrGen;
using V3d = V3<double>;

// One instance with loop closures inside a kernel. save/delta are column
// planes that are free between integrator steps (entry q/u of a projection,
// the last correction).
struct LoopState {
    const DevTables& T;
    int inst;
    SC64 S;
    double* y;
    double* save;
    double* delta;
    int64_t base, stride;
    bool rows;  // level-parallel layout: record = local row, slots after the bodies
    int body0, nb;
    // record of body row `row`, slot record of a loop body row
    __device__ __forceinline__ int rec(int row) const { return rows ? row - body0 : T.srec[row]; }
    __device__ __forceinline__ int slot(int row) const { return rows ? nb + T.lslot[row] : T.lrec[row]; }
};
// The state of instance `inst` over records at `scratch` (its record base):
// one-thread layout with stride s, or the level-parallel layout.
__device__ __forceinline__ LoopState loopStateChain(const DevTables& T, int inst, double* scratch, int s, double* y,
                                                    double* save, double* delta, int64_t base, int64_t stride) {
    return LoopState{T, inst, SC64{scratch, s, s}, y, save, delta, base, stride, false, T.ibody[inst], T.inb[inst]};
}
// The level-parallel layout of an instance with loop closures: one record
// per row (the bodies, then 2 slot records per constraint), record-major
// with the record width in T.sstride (element f of row r at r * W + f).
__device__ __forceinline__ int loopRows(const DevTables& T, int inst) { return T.inb[inst] + 2 * T.incons[inst]; }
__device__ __forceinline__ LoopState loopStateRows(const DevTables& T, int inst, double* scratch, double* y,
                                                   double* save, double* delta, int64_t base, int64_t stride) {
    return LoopState{T, inst, SC64{scratch, (int)T.sstride[inst], 1}, y, save, delta, base, stride, true,
                     T.ibody[inst], T.inb[inst]};
}

// The weights of a sweep that applies none (kMInvSweep; see PosWeights).
struct NoWeights {
    __device__ __forceinline__ void apply(int, int, double*) const {}
};

struct NullOut {
    template <class R> __device__ __forceinline__ void qdot(int, R) {}
    template <class R> __device__ __forceinline__ void udot(int, R) {}
};

enum : int { kMInvSweep = 0, kJacSweep = 1 };

__device__ __forceinline__ int recN(int n, int NM) { return n == 6 ? 6 : NM; }
__device__ __forceinline__ int recEps(int N) { return kRecH + 6 * N + N + N * N + 6 * N; }

// Position and velocity kinematics of the state in y (pass 1 only): body
// records (H, l, ...) and the slot records of the constrained bodies.
template <int NM>
__device__ __noinline__ void loopKinematics(const LoopState& L) {
    const DevTables& T = L.T;
    const int body0 = T.ibody[L.inst], nb = T.inb[L.inst];
    const YSrc src{L.y, L.base, L.stride, T.inq[L.inst]};
    NullOut out;
    const V3d g = mk3(T.grav[3 * L.inst], T.grav[3 * L.inst + 1], T.grav[3 * L.inst + 2]);
    Kin<double> carry = groundKin<double>();
    for (int lb = 0; lb < nb; ++lb) {
        const int row = body0 + lb;
        const int info = T.info[row];
        if (!(info & F_LOOPPATH)) continue;  // a path row's parent is a path row
        const int parent = T.parent[row];
        const int rec = L.rec(row);
        const Kin<double> P = parent < 0 ? groundKin<double>()
                              : (info & F_CARRY) ? carry : loadKin<double>(L.S, L.rec(body0 + parent));
        carry = body1<double, NM>(T, row, rec, L.S, src, out, g, P);
        if (info & F_MEMCHILD) storeKin(L.S, rec, carry);
        if (info & F_LOOPBODY) storeKin(L.S, L.slot(row), carry);
    }
}

struct LoopGeom {
    V3d pS, pP, r1, r2;  // S and P in Ground; S relative to the origins of body 1 and body 2
    int s1, s2;          // slot records (-1 = Ground)
};

__device__ __forceinline__ void loopSlots(const LoopState& L, int c, int& s1, int& s2) {
    const DevTables& T = L.T;
    const int gc = T.icons[L.inst] + c, body0 = T.ibody[L.inst];
    const int r1 = T.lcons[2 * gc], r2 = T.lcons[2 * gc + 1];
    s1 = r1 >= 0 ? L.slot(body0 + r1) : -1;
    s2 = r2 >= 0 ? L.slot(body0 + r2) : -1;
}

__device__ __forceinline__ LoopGeom loopGeom(const LoopState& L, int c) {
    LoopGeom G;
    loopSlots(L, c, G.s1, G.s2);
    const double* st = L.T.lst + 6 * (int64_t)(L.T.icons[L.inst] + c);
    const V3d st1 = mk3(st[0], st[1], st[2]), st2 = mk3(st[3], st[4], st[5]);
    if (G.s2 >= 0) {
        const Kin<double> K = loadKin<double>(L.S, G.s2);
        G.r2 = mul(K.R_, st2);
        G.pS = K.p + G.r2;
    } else {
        G.r2 = z3<double>();
        G.pS = st2;
    }
    if (G.s1 >= 0) {
        const Kin<double> K = loadKin<double>(L.S, G.s1);
        G.pP = K.p + mul(K.R_, st1);
        G.r1 = G.pS - K.p;
    } else {
        G.pP = st1;
        G.r1 = z3<double>();
    }
    return G;
}

// Linear part of a spatial vector (angular at f, linear at f+3) moved to
// the material point at offset r: x_v + x_w x r.
__device__ __forceinline__ V3d slotPoint(const SC64& S, int slot, int f, V3d r) {
    if (slot < 0) return z3<double>();
    return ld3<double>(S, slot, f + 3) + cross(ld3<double>(S, slot, f), r);
}
__device__ __forceinline__ V3d slotCentripetal(const SC64& S, int slot, V3d r) {
    if (slot < 0) return z3<double>();
    const V3d w = ld3<double>(S, slot, 12);
    return cross(w, cross(w, r));
}

__device__ __forceinline__ void loopClearForces(const LoopState& L) {
    const int nc = L.T.incons[L.inst];
    for (int c = 0; c < nc; ++c) {
        int s1, s2;
        loopSlots(L, c, s1, s2);
        if (s1 >= 0) { st3<double>(L.S, s1, kSlotF, z3<double>()); st3<double>(L.S, s1, kSlotF + 3, z3<double>()); }
        if (s2 >= 0) { st3<double>(L.S, s2, kSlotF, z3<double>()); st3<double>(L.S, s2, kSlotF + 3, z3<double>()); }
    }
}
// Point force F at offset r from the body origin, as (r x F, F) at the origin.
__device__ __forceinline__ void loopAddForce(const SC64& S, int slot, V3d r, V3d F) {
    if (slot < 0) return;
    st3<double>(S, slot, kSlotF, ld3<double>(S, slot, kSlotF) + cross(r, F));
    st3<double>(S, slot, kSlotF + 3, ld3<double>(S, slot, kSlotF + 3) + F);
}
// +x at S on body 2, -x at C on body 1 (the forces of G^T x for constraint c).
__device__ __forceinline__ void loopAddConstraintForce(const LoopState& L, const LoopGeom& G, V3d x) {
    loopAddForce(L.S, G.s2, G.r2, x);
    loopAddForce(L.S, G.s1, G.r1, -x);
}

// Inward half for one body; (zw, zv): in, the children's sum at the body
// origin; out, the contribution to the parent.
//   kMInvSweep: z = children - F, eps = -~H z (stored), z+ = z + G eps
//               (RigidBodyNodeSpec.cpp:483-515 with f = 0)
//   kJacSweep:  F = children + F_applied, g = ~H F (stored), F passed on
template <int N, int KIND>
__device__ __forceinline__ void loopIn(const LoopState& L, int row, int rec, int n, int info, V3d& zw, V3d& zv) {
    const SC64& S = L.S;
    const int eDI = kRecH + 7 * N, eG = eDI + N * N, eEps = eG + 6 * N;
    if (info & F_LOOPBODY) {
        const int sl = L.slot(row);
        const V3d tw = ld3<double>(S, sl, kSlotF), tv = ld3<double>(S, sl, kSlotF + 3);
        if (KIND == kMInvSweep) { zw = zw - tw; zv = zv - tv; }
        else { zw = zw + tw; zv = zv + tv; }
    }
    V3d pw = zw, pv = zv;
#pragma unroll
    for (int j = 0; j < N; ++j) {
        if (j < n) {
            const double d = dot(ld3<double>(S, rec, kRecH + 6 * j), zw) + dot(ld3<double>(S, rec, kRecH + 6 * j + 3), zv);
            if (KIND == kMInvSweep) {
                const double eps = -d;
                S(rec, eEps + j) = eps;
                pw = axpy(pw, eps, ld3<double>(S, rec, eG + 6 * j));
                pv = axpy(pv, eps, ld3<double>(S, rec, eG + 6 * j + 3));
            } else {
                S(rec, eEps + j) = d;
            }
        }
    }
    const V3d l = ld3<double>(S, rec, kRecL);
    zw = pw + cross(l, pv);
    zv = pv;
}

// Outward half for one body; (Aw, Av): in, the parent's value; out, this
// body's. ud gets the body's mobility values.
//   kMInvSweep: udot = DI eps - ~G A+, A = A+ + H udot (a = 0)
//               (RigidBodyNodeSpec.cpp:517-552)
//   kJacSweep:  du = the stored (weighted) values, V = V+ + H du
template <int N, int KIND>
__device__ __forceinline__ void loopOut(const LoopState& L, int rec, int n, bool hasParent, bool onPath, V3d& Aw,
                                        V3d& Av, double* ud) {
    const SC64& S = L.S;
    const int eDI = kRecH + 7 * N, eG = eDI + N * N, eEps = eG + 6 * N;
    const V3d l = ld3<double>(S, rec, kRecL);
    const V3d Apw = hasParent ? Aw : z3<double>();
    const V3d Apv = hasParent ? Av + cross(Aw, l) : z3<double>();
    double eps[N];
#pragma unroll
    for (int j = 0; j < N; ++j) eps[j] = j < n && onPath ? S(rec, eEps + j) : 0.0;
    Aw = Apw;
    Av = Apv;
#pragma unroll
    for (int i = 0; i < N; ++i) {
        if (i < n) {
            double s;
            if (KIND == kMInvSweep) {
                s = 0.0;
#pragma unroll
                for (int k = 0; k < N; ++k)
                    if (k < n) s = s + S(rec, eDI + i * N + k) * eps[k];
                s = s - (dot(ld3<double>(S, rec, eG + 6 * i), Apw) + dot(ld3<double>(S, rec, eG + 6 * i + 3), Apv));
            } else {
                s = eps[i];
            }
            ud[i] = s;
            Aw = axpy(Aw, s, ld3<double>(S, rec, kRecH + 6 * i));
            Av = axpy(Av, s, ld3<double>(S, rec, kRecH + 6 * i + 3));
        }
    }
}

template <int KIND>
__device__ __noinline__ void loopIn6(const LoopState& L, int row, int rec, int info, V3d& zw, V3d& zv) {
    loopIn<6, KIND>(L, row, rec, 6, info, zw, zv);
}
template <int KIND>
__device__ __noinline__ void loopOut6(const LoopState& L, int rec, bool hasParent, bool onPath, V3d& Aw, V3d& Av,
                                      double* ud) {
    loopOut<6, KIND>(L, rec, 6, hasParent, onPath, Aw, Av, ud);
}

// Children's sums of the inward sweeps live in the z accumulator of the
// parent's record; it is read and cleared by the parent. Tree passes (and
// fresh memory) leave other values there, so every entry point that starts
// a series of sweeps clears them first.
__device__ __forceinline__ void loopZeroAcc(const LoopState& L) {
    const DevTables& T = L.T;
    const int body0 = T.ibody[L.inst], nb = T.inb[L.inst];
    for (int lb = 0; lb < nb; ++lb) {
        const int row = body0 + lb;
        if ((T.info[row] & (F_MEMCHILD | F_LOOPPATH)) == (F_MEMCHILD | F_LOOPPATH)) {
            st3<double>(L.S, L.rec(row), kRecZacc, z3<double>());
            st3<double>(L.S, L.rec(row), kRecZacc + 3, z3<double>());
        }
    }
}

// Inward half of a sweep driven by the applied forces in the slot records
// (path rows only: the others contribute zero). kJacSweep multiplies g by
// wt(row, j) after the body's step.
template <int NM, int KIND, class Wt>
__device__ __forceinline__ void loopSweepIn(const LoopState& L, const Wt& wt) {
    const DevTables& T = L.T;
    const SC64& S = L.S;
    const int body0 = T.ibody[L.inst], nb = T.inb[L.inst];
    V3d cw = z3<double>(), cv = z3<double>();
    bool have = false;
    for (int lb = nb - 1; lb >= 0; --lb) {
        const int row = body0 + lb;
        const int info = T.info[row];
        if (!(info & F_LOOPPATH)) {  // contributes zero
            have = false;
            continue;
        }
        const int n = (info >> 4) & 15;
        const int rec = L.rec(row);
        V3d zw = z3<double>(), zv = z3<double>();
        if (info & F_MEMCHILD) {
            zw = ld3<double>(S, rec, kRecZacc);
            zv = ld3<double>(S, rec, kRecZacc + 3);
            st3<double>(S, rec, kRecZacc, z3<double>());
            st3<double>(S, rec, kRecZacc + 3, z3<double>());
        }
        if (have) { zw = zw + cw; zv = zv + cv; }
        if (n == 6) loopIn6<KIND>(L, row, rec, info, zw, zv);
        else loopIn<NM, KIND>(L, row, rec, n, info, zw, zv);
        if constexpr (KIND == kJacSweep) {
            const int eEps = recEps(recN(n, NM));
            double g[6];
            for (int j = 0; j < n; ++j) g[j] = S(rec, eEps + j);
            wt.apply(row, n, g);
            for (int j = 0; j < n; ++j) S(rec, eEps + j) = g[j];
        }
        const int parent = T.parent[row];
        have = (info & F_CARRY) != 0;
        if (have) {
            cw = zw;
            cv = zv;
        } else if (parent >= 0) {
            const int pr = L.rec(body0 + parent);
            st3<double>(S, pr, kRecZacc, ld3<double>(S, pr, kRecZacc) + zw);
            st3<double>(S, pr, kRecZacc + 3, ld3<double>(S, pr, kRecZacc + 3) + zv);
        }
    }
}

// Outward half. The outward result of each constrained body goes to its
// slot (kSlotB); onBody(row, n, ud) sees the mobility values of every path
// row (of every row with FULL_OUT, which take zero eps off the paths).
template <int NM, int KIND, bool FULL_OUT, class OnBody>
__device__ __forceinline__ void loopSweepOut(const LoopState& L, const OnBody& onBody) {
    const DevTables& T = L.T;
    const SC64& S = L.S;
    const int body0 = T.ibody[L.inst], nb = T.inb[L.inst];
    V3d aw = z3<double>(), av = z3<double>();
    for (int lb = 0; lb < nb; ++lb) {
        const int row = body0 + lb;
        const int info = T.info[row];
        const bool onPath = (info & F_LOOPPATH) != 0;
        if (!FULL_OUT && !onPath) continue;  // a path row's parent is a path row
        const int n = (info >> 4) & 15;
        const int rec = L.rec(row);
        const int parent = T.parent[row];
        const bool hp = parent >= 0;
        V3d pw = aw, pv = av;
        if (hp && !(info & F_CARRY)) {
            const int pr = L.rec(body0 + parent);
            pw = ld3<double>(S, pr, 0);
            pv = ld3<double>(S, pr, 3);
        }
        double ud[6];
        if (n == 6) loopOut6<KIND>(L, rec, hp, onPath, pw, pv, ud);
        else loopOut<NM, KIND>(L, rec, n, hp, onPath, pw, pv, ud);
        onBody(row, n, ud);
        if (info & F_LOOPBODY) {
            st3<double>(S, L.slot(row), kSlotB, pw);
            st3<double>(S, L.slot(row), kSlotB + 3, pv);
        }
        if (info & F_MEMCHILD) {
            st3<double>(S, rec, 0, pw);
            st3<double>(S, rec, 3, pv);
        }
        aw = pw;
        av = pv;
    }
}

// One inward and one outward sweep over the instance.
template <int NM, int KIND, bool FULL_OUT = false, class Wt, class OnBody>
__device__ __forceinline__ void loopSweep(const LoopState& L, const Wt& wt, const OnBody& onBody) {
    loopSweepIn<NM, KIND>(L, wt);
    loopSweepOut<NM, KIND, FULL_OUT>(L, onBody);
}

// -------------------------------------------- three Gram columns per sweep
// The three columns of one Ball constraint (unit forces along x, y, z at the
// same two points) share one sweep: each row's data is loaded once and its
// step runs once per column, with each column's arithmetic exactly that of
// the single-column sweep. Column 0 keeps its values where the single-column
// sweep does; columns 1 and 2 use fields the tree passes have finished with
// (the next RHS or kinematics pass refills them):
//   slot record   F_k (applied force), B_k (outward result)
//   body record   eps_k, the z accumulator and the outward acceleration
__device__ __forceinline__ int slotF(int k) { return k == 0 ? kSlotF : kSlotF3 + 6 * (k - 1); }
__device__ __forceinline__ int slotB(int k) { return k == 0 ? kSlotB : kSlotB3 + 6 * (k - 1); }
__device__ __forceinline__ int recEpsK(int eEps, int k) { return k == 0 ? eEps : kRecA + 6 * (k - 1); }
__device__ __forceinline__ int recZaccK(int k) { return k == 0 ? kRecZacc : (k == 1 ? kRecPc : kRecPacc); }

__device__ __forceinline__ void loopZeroAcc3(const LoopState& L) {
    const DevTables& T = L.T;
    const int body0 = T.ibody[L.inst], nb = T.inb[L.inst];
    for (int lb = 0; lb < nb; ++lb) {
        const int row = body0 + lb;
        if ((T.info[row] & (F_MEMCHILD | F_LOOPPATH)) == (F_MEMCHILD | F_LOOPPATH))
            for (int k = 0; k < 3; ++k) {
                st3<double>(L.S, L.rec(row), recZaccK(k), z3<double>());
                st3<double>(L.S, L.rec(row), recZaccK(k) + 3, z3<double>());
            }
    }
}
__device__ __forceinline__ void loopClearForces3(const LoopState& L) {
    const int nc = L.T.incons[L.inst];
    for (int c = 0; c < nc; ++c) {
        int s1, s2;
        loopSlots(L, c, s1, s2);
        for (int k = 0; k < 3; ++k) {
            if (s1 >= 0) { st3<double>(L.S, s1, slotF(k), z3<double>()); st3<double>(L.S, s1, slotF(k) + 3, z3<double>()); }
            if (s2 >= 0) { st3<double>(L.S, s2, slotF(k), z3<double>()); st3<double>(L.S, s2, slotF(k) + 3, z3<double>()); }
        }
    }
}
__device__ __forceinline__ void loopAddForceK(const SC64& S, int slot, V3d r, V3d F, int k) {
    if (slot < 0) return;
    st3<double>(S, slot, slotF(k), ld3<double>(S, slot, slotF(k)) + cross(r, F));
    st3<double>(S, slot, slotF(k) + 3, ld3<double>(S, slot, slotF(k) + 3) + F);
}

template <int N, int KIND>
__device__ __forceinline__ void loopIn3(const LoopState& L, int row, int rec, int n, int info, V3d* zw, V3d* zv) {
    const SC64& S = L.S;
    const int eDI = kRecH + 7 * N, eG = eDI + N * N, eEps = eG + 6 * N;
    if (info & F_LOOPBODY) {
        const int sl = L.slot(row);
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const V3d tw = ld3<double>(S, sl, slotF(k)), tv = ld3<double>(S, sl, slotF(k) + 3);
            if (KIND == kMInvSweep) { zw[k] = zw[k] - tw; zv[k] = zv[k] - tv; }
            else { zw[k] = zw[k] + tw; zv[k] = zv[k] + tv; }
        }
    }
    V3d pw[3] = {zw[0], zw[1], zw[2]}, pv[3] = {zv[0], zv[1], zv[2]};
#pragma unroll
    for (int j = 0; j < N; ++j) {
        if (j < n) {
            const V3d hw = ld3<double>(S, rec, kRecH + 6 * j), hv = ld3<double>(S, rec, kRecH + 6 * j + 3);
            V3d gw = z3<double>(), gv = z3<double>();
            if (KIND == kMInvSweep) { gw = ld3<double>(S, rec, eG + 6 * j); gv = ld3<double>(S, rec, eG + 6 * j + 3); }
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                const double d = dot(hw, zw[k]) + dot(hv, zv[k]);
                if (KIND == kMInvSweep) {
                    const double eps = -d;
                    S(rec, recEpsK(eEps, k) + j) = eps;
                    pw[k] = axpy(pw[k], eps, gw);
                    pv[k] = axpy(pv[k], eps, gv);
                } else {
                    S(rec, recEpsK(eEps, k) + j) = d;
                }
            }
        }
    }
    const V3d l = ld3<double>(S, rec, kRecL);
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        zw[k] = pw[k] + cross(l, pv[k]);
        zv[k] = pv[k];
    }
}

template <int N, int KIND>
__device__ __forceinline__ void loopOut3(const LoopState& L, int rec, int n, bool hasParent, V3d* Aw, V3d* Av) {
    const SC64& S = L.S;
    const int eDI = kRecH + 7 * N, eG = eDI + N * N, eEps = eG + 6 * N;
    const V3d l = ld3<double>(S, rec, kRecL);
    V3d Apw[3], Apv[3];
    double eps[3][N];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        Apw[k] = hasParent ? Aw[k] : z3<double>();
        Apv[k] = hasParent ? Av[k] + cross(Aw[k], l) : z3<double>();
#pragma unroll
        for (int j = 0; j < N; ++j) eps[k][j] = j < n ? S(rec, recEpsK(eEps, k) + j) : 0.0;
        Aw[k] = Apw[k];
        Av[k] = Apv[k];
    }
#pragma unroll
    for (int i = 0; i < N; ++i) {
        if (i < n) {
            const V3d hw = ld3<double>(S, rec, kRecH + 6 * i), hv = ld3<double>(S, rec, kRecH + 6 * i + 3);
            V3d gw = z3<double>(), gv = z3<double>();
            if (KIND == kMInvSweep) { gw = ld3<double>(S, rec, eG + 6 * i); gv = ld3<double>(S, rec, eG + 6 * i + 3); }
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                double s;
                if (KIND == kMInvSweep) {
                    s = 0.0;
#pragma unroll
                    for (int c = 0; c < N; ++c)
                        if (c < n) s = s + S(rec, eDI + i * N + c) * eps[k][c];
                    s = s - (dot(gw, Apw[k]) + dot(gv, Apv[k]));
                } else {
                    s = eps[k][i];
                }
                Aw[k] = axpy(Aw[k], s, hw);
                Av[k] = axpy(Av[k], s, hv);
            }
        }
    }
}

template <int KIND>
__device__ __noinline__ void loopIn36(const LoopState& L, int row, int rec, int info, V3d* zw, V3d* zv) {
    loopIn3<6, KIND>(L, row, rec, 6, info, zw, zv);
}
template <int KIND>
__device__ __noinline__ void loopOut36(const LoopState& L, int rec, bool hasParent, V3d* Aw, V3d* Av) {
    loopOut3<6, KIND>(L, rec, 6, hasParent, Aw, Av);
}

// The three-column sweep over the loop-path rows: inward, then outward with
// the constrained bodies' results in their slots (B_k).
template <int NM, int KIND, class Wt>
__device__ __forceinline__ void loopSweep3(const LoopState& L, const Wt& wt) {
    const DevTables& T = L.T;
    const SC64& S = L.S;
    const int body0 = T.ibody[L.inst], nb = T.inb[L.inst];
    {
        V3d cw[3], cv[3];
        bool have = false;
        for (int lb = nb - 1; lb >= 0; --lb) {
            const int row = body0 + lb;
            const int info = T.info[row];
            if (!(info & F_LOOPPATH)) {
                have = false;
                continue;
            }
            const int n = (info >> 4) & 15;
            const int rec = L.rec(row);
            V3d zw[3], zv[3];
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                zw[k] = z3<double>();
                zv[k] = z3<double>();
                if (info & F_MEMCHILD) {
                    zw[k] = ld3<double>(S, rec, recZaccK(k));
                    zv[k] = ld3<double>(S, rec, recZaccK(k) + 3);
                    st3<double>(S, rec, recZaccK(k), z3<double>());
                    st3<double>(S, rec, recZaccK(k) + 3, z3<double>());
                }
                if (have) { zw[k] = zw[k] + cw[k]; zv[k] = zv[k] + cv[k]; }
            }
            if (n == 6) loopIn36<KIND>(L, row, rec, info, zw, zv);
            else loopIn3<NM, KIND>(L, row, rec, n, info, zw, zv);
            if constexpr (KIND == kJacSweep) {
                const int eEps = recEps(recN(n, NM));
                for (int k = 0; k < 3; ++k) {
                    double g[6];
                    for (int j = 0; j < n; ++j) g[j] = S(rec, recEpsK(eEps, k) + j);
                    wt.apply(row, n, g);
                    for (int j = 0; j < n; ++j) S(rec, recEpsK(eEps, k) + j) = g[j];
                }
            }
            const int parent = T.parent[row];
            have = (info & F_CARRY) != 0;
            if (have) {
#pragma unroll
                for (int k = 0; k < 3; ++k) { cw[k] = zw[k]; cv[k] = zv[k]; }
            } else if (parent >= 0) {
                const int pr = L.rec(body0 + parent);
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    st3<double>(S, pr, recZaccK(k), ld3<double>(S, pr, recZaccK(k)) + zw[k]);
                    st3<double>(S, pr, recZaccK(k) + 3, ld3<double>(S, pr, recZaccK(k) + 3) + zv[k]);
                }
            }
        }
    }
    {
        V3d aw[3], av[3];
        for (int k = 0; k < 3; ++k) { aw[k] = z3<double>(); av[k] = z3<double>(); }
        for (int lb = 0; lb < nb; ++lb) {
            const int row = body0 + lb;
            const int info = T.info[row];
            if (!(info & F_LOOPPATH)) continue;
            const int n = (info >> 4) & 15;
            const int rec = L.rec(row);
            const int parent = T.parent[row];
            const bool hp = parent >= 0;
            V3d pw[3], pv[3];
#pragma unroll
            for (int k = 0; k < 3; ++k) { pw[k] = aw[k]; pv[k] = av[k]; }
            if (hp && !(info & F_CARRY)) {
                const int pr = L.rec(body0 + parent);
#pragma unroll
                for (int k = 0; k < 3; ++k) { pw[k] = ld3<double>(S, pr, 6 * k); pv[k] = ld3<double>(S, pr, 6 * k + 3); }
            }
            if (n == 6) loopOut36<KIND>(L, rec, hp, pw, pv);
            else loopOut3<NM, KIND>(L, rec, n, hp, pw, pv);
            if (info & F_LOOPBODY)
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    st3<double>(S, L.slot(row), slotB(k), pw[k]);
                    st3<double>(S, L.slot(row), slotB(k) + 3, pv[k]);
                }
            if (info & F_MEMCHILD)
#pragma unroll
                for (int k = 0; k < 3; ++k) { st3<double>(S, rec, 6 * k, pw[k]); st3<double>(S, rec, 6 * k + 3, pv[k]); }
#pragma unroll
            for (int k = 0; k < 3; ++k) { aw[k] = pw[k]; av[k] = pv[k]; }
        }
    }
}

// ----------------------------------------- one Gram column per group lane
// The same sweep with lane k of a request's group (k < 3) taking column k
// alone: column k's arithmetic and fields are those of the three-column
// sweep, and no column reads another's fields, so the three lanes run side
// by side with the three-column sweep's results bit for bit. An FP64 warp
// instruction occupies the FP64 pipe alike for one active lane or for three,
// so on the FP64-poor GB300 this cuts the Gram's time about threefold.
template <int N, int KIND>
__device__ __forceinline__ void loopIn1(const LoopState& L, int row, int rec, int n, int info, int k, V3d& zw, V3d& zv) {
    const SC64& S = L.S;
    const int eDI = kRecH + 7 * N, eG = eDI + N * N, eEps = eG + 6 * N;
    const int fE = recEpsK(eEps, k);
    if (info & F_LOOPBODY) {
        const int sl = L.slot(row);
        const V3d tw = ld3<double>(S, sl, slotF(k)), tv = ld3<double>(S, sl, slotF(k) + 3);
        if (KIND == kMInvSweep) { zw = zw - tw; zv = zv - tv; }
        else { zw = zw + tw; zv = zv + tv; }
    }
    V3d pw = zw, pv = zv;
#pragma unroll
    for (int j = 0; j < N; ++j) {
        if (j < n) {
            const V3d hw = ld3<double>(S, rec, kRecH + 6 * j), hv = ld3<double>(S, rec, kRecH + 6 * j + 3);
            const double d = dot(hw, zw) + dot(hv, zv);
            if (KIND == kMInvSweep) {
                const V3d gw = ld3<double>(S, rec, eG + 6 * j), gv = ld3<double>(S, rec, eG + 6 * j + 3);
                const double eps = -d;
                S(rec, fE + j) = eps;
                pw = axpy(pw, eps, gw);
                pv = axpy(pv, eps, gv);
            } else {
                S(rec, fE + j) = d;
            }
        }
    }
    const V3d l = ld3<double>(S, rec, kRecL);
    zw = pw + cross(l, pv);
    zv = pv;
}

template <int N, int KIND>
__device__ __forceinline__ void loopOut1(const LoopState& L, int rec, int n, bool hasParent, int k, V3d& Aw, V3d& Av) {
    const SC64& S = L.S;
    const int eDI = kRecH + 7 * N, eG = eDI + N * N, eEps = eG + 6 * N;
    const int fE = recEpsK(eEps, k);
    const V3d l = ld3<double>(S, rec, kRecL);
    const V3d Apw = hasParent ? Aw : z3<double>();
    const V3d Apv = hasParent ? Av + cross(Aw, l) : z3<double>();
    double eps[N];
#pragma unroll
    for (int j = 0; j < N; ++j) eps[j] = j < n ? S(rec, fE + j) : 0.0;
    Aw = Apw;
    Av = Apv;
#pragma unroll
    for (int i = 0; i < N; ++i) {
        if (i < n) {
            const V3d hw = ld3<double>(S, rec, kRecH + 6 * i), hv = ld3<double>(S, rec, kRecH + 6 * i + 3);
            double sv;
            if (KIND == kMInvSweep) {
                const V3d gw = ld3<double>(S, rec, eG + 6 * i), gv = ld3<double>(S, rec, eG + 6 * i + 3);
                sv = 0.0;
#pragma unroll
                for (int c = 0; c < N; ++c)
                    if (c < n) sv = sv + S(rec, eDI + i * N + c) * eps[c];
                sv = sv - (dot(gw, Apw) + dot(gv, Apv));
            } else {
                sv = eps[i];
            }
            Aw = axpy(Aw, sv, hw);
            Av = axpy(Av, sv, hv);
        }
    }
}

template <int KIND>
__device__ __noinline__ void loopIn16(const LoopState& L, int row, int rec, int info, int k, V3d& zw, V3d& zv) {
    loopIn1<6, KIND>(L, row, rec, 6, info, k, zw, zv);
}
template <int KIND>
__device__ __noinline__ void loopOut16(const LoopState& L, int rec, bool hasParent, int k, V3d& Aw, V3d& Av) {
    loopOut1<6, KIND>(L, rec, 6, hasParent, k, Aw, Av);
}

// Column k of the three-column sweep (loopSweep3), on one lane.
template <int NM, int KIND, class Wt>
__device__ __forceinline__ void loopSweepColumn(const LoopState& L, const Wt& wt, int k) {
    const DevTables& T = L.T;
    const SC64& S = L.S;
    const int body0 = T.ibody[L.inst], nb = T.inb[L.inst];
    const int fZ = recZaccK(k);
    {
        V3d cw = z3<double>(), cv = z3<double>();
        bool have = false;
        for (int lb = nb - 1; lb >= 0; --lb) {
            const int row = body0 + lb;
            const int info = T.info[row];
            if (!(info & F_LOOPPATH)) {
                have = false;
                continue;
            }
            const int n = (info >> 4) & 15;
            const int rec = L.rec(row);
            V3d zw = z3<double>(), zv = z3<double>();
            if (info & F_MEMCHILD) {
                zw = ld3<double>(S, rec, fZ);
                zv = ld3<double>(S, rec, fZ + 3);
                st3<double>(S, rec, fZ, z3<double>());
                st3<double>(S, rec, fZ + 3, z3<double>());
            }
            if (have) { zw = zw + cw; zv = zv + cv; }
            if (n == 6) loopIn16<KIND>(L, row, rec, info, k, zw, zv);
            else loopIn1<NM, KIND>(L, row, rec, n, info, k, zw, zv);
            if constexpr (KIND == kJacSweep) {
                const int fE = recEpsK(recEps(recN(n, NM)), k);
                double g[6];
                for (int j = 0; j < n; ++j) g[j] = S(rec, fE + j);
                wt.apply(row, n, g);
                for (int j = 0; j < n; ++j) S(rec, fE + j) = g[j];
            }
            const int parent = T.parent[row];
            have = (info & F_CARRY) != 0;
            if (have) {
                cw = zw;
                cv = zv;
            } else if (parent >= 0) {
                const int pr = L.rec(body0 + parent);
                st3<double>(S, pr, fZ, ld3<double>(S, pr, fZ) + zw);
                st3<double>(S, pr, fZ + 3, ld3<double>(S, pr, fZ + 3) + zv);
            }
        }
    }
    {
        V3d aw = z3<double>(), av = z3<double>();
        for (int lb = 0; lb < nb; ++lb) {
            const int row = body0 + lb;
            const int info = T.info[row];
            if (!(info & F_LOOPPATH)) continue;
            const int n = (info >> 4) & 15;
            const int rec = L.rec(row);
            const int parent = T.parent[row];
            const bool hp = parent >= 0;
            V3d pw = aw, pv = av;
            if (hp && !(info & F_CARRY)) {
                const int pr = L.rec(body0 + parent);
                pw = ld3<double>(S, pr, 6 * k);
                pv = ld3<double>(S, pr, 6 * k + 3);
            }
            if (n == 6) loopOut16<KIND>(L, rec, hp, k, pw, pv);
            else loopOut1<NM, KIND>(L, rec, n, hp, k, pw, pv);
            if (info & F_LOOPBODY) {
                st3<double>(S, L.slot(row), slotB(k), pw);
                st3<double>(S, L.slot(row), slotB(k) + 3, pv);
            }
            if (info & F_MEMCHILD) { st3<double>(S, rec, 6 * k, pw); st3<double>(S, rec, 6 * k + 3, pv); }
            aw = pw;
            av = pv;
        }
    }
}

// Rank-revealing Cholesky of the leading m x m block of a positive
// semidefinite Gram (row stride kMaxLoopEq; its lower triangle is the matrix):
// symmetric pivoting, the largest remaining diagonal first, stopping at the
// first pivot not above relTol times the first. F.r is the rank kept and
// F.piv the order of the equations: A = W W^T with W = P [L11; L21] (m x r).
// loopCholSolve gives the least-squares solution lambda = W (W^T W)^-2 W^T b
// (A^-1 b at full rank). The reference's QTZ factorization takes the
// minimum-norm least-squares solution; the two differ by a null vector of A,
// which is one of G^T, so the constraint forces and the projections'
// corrections agree, also where the equations of redundant closures do not
// (the centripetal accelerations of two pinned points of one body spinning
// about another axis). relTol is the reference's conditioning tolerance for
// the matrix the Gram squares: kAccRelTol for G M^-1 G^T, whose own
// condition the reference tests, kProjRelTol for G D G^T, the square of the
// weighted Jacobian whose condition it tests. false when the block is not
// finite or its largest diagonal is not positive.
struct LoopFactor {
    int r;
    signed char piv[kMaxLoopEq];
};
__device__ __forceinline__ double kAccRelTol(int m) { return m * 1.8189894035458565e-12; }  // m Eps^(3/4)
__device__ __forceinline__ double kProjRelTol(int m) { return (double)(m * m) * 2.220446049250313e-16; }  // (m Eps^(1/2))^2

__device__ __forceinline__ bool loopCholFactor(int m, double* A, double relTol, LoopFactor& F) {
    F.r = 0;
    for (int i = 0; i < m; ++i) {
        F.piv[i] = (signed char)i;
        for (int k = 0; k <= i; ++k) {
            const double v = A[i * kMaxLoopEq + k];
            if (!isfinite(v)) return false;
            A[k * kMaxLoopEq + i] = v;
        }
    }
    double d0 = 0;
    for (int j = 0; j < m; ++j) {
        int p = j;
        double best = A[j * kMaxLoopEq + j];
        for (int i = j + 1; i < m; ++i)
            if (A[i * kMaxLoopEq + i] > best) { best = A[i * kMaxLoopEq + i]; p = i; }
        if (j == 0) {
            if (!(best > 0)) return false;
            d0 = best;
        }
        if (!(best > relTol * d0)) break;
        if (p != j) {
            for (int k = 0; k < m; ++k) {
                const double t = A[j * kMaxLoopEq + k];
                A[j * kMaxLoopEq + k] = A[p * kMaxLoopEq + k];
                A[p * kMaxLoopEq + k] = t;
            }
            for (int k = 0; k < m; ++k) {
                const double t = A[k * kMaxLoopEq + j];
                A[k * kMaxLoopEq + j] = A[k * kMaxLoopEq + p];
                A[k * kMaxLoopEq + p] = t;
            }
            const signed char t = F.piv[j];
            F.piv[j] = F.piv[p];
            F.piv[p] = t;
        }
        const double d = sqrt(best);
        A[j * kMaxLoopEq + j] = d;
        for (int i = j + 1; i < m; ++i) A[i * kMaxLoopEq + j] /= d;
        for (int i = j + 1; i < m; ++i)
            for (int k = j + 1; k < m; ++k) A[i * kMaxLoopEq + k] -= A[i * kMaxLoopEq + j] * A[k * kMaxLoopEq + j];
        F.r = j + 1;
    }
    return true;
}
__device__ __forceinline__ void loopCholSolve(int m, const double* A, const LoopFactor& F, double* b) {
    double w[kMaxLoopEq];
    for (int i = 0; i < m; ++i) w[i] = b[F.piv[i]];
    const int r = F.r;
    if (r == m) {
        for (int i = 0; i < r; ++i) {
            double v = w[i];
            for (int k = 0; k < i; ++k) v -= A[i * kMaxLoopEq + k] * w[k];
            w[i] = v / A[i * kMaxLoopEq + i];
        }
        for (int i = r - 1; i >= 0; --i) {
            double v = w[i];
            for (int k = i + 1; k < r; ++k) v -= A[k * kMaxLoopEq + i] * w[k];
            w[i] = v / A[i * kMaxLoopEq + i];
        }
        for (int i = 0; i < m; ++i) b[F.piv[i]] = w[i];
        return;
    }
    // W[i][j] = A[i][j] for i >= j, j < r. C = W^T W = R R^T (lower R);
    // y = C^-1 C^-1 W^T w; lambda = W y.
    double C[kMaxLoopEq * kMaxLoopEq], y[kMaxLoopEq];
    for (int j = 0; j < r; ++j) {
        double t = 0;
        for (int i = j; i < m; ++i) t += A[i * kMaxLoopEq + j] * w[i];
        y[j] = t;
        for (int k = 0; k <= j; ++k) {
            double c = 0;
            for (int i = j; i < m; ++i) c += A[i * kMaxLoopEq + j] * A[i * kMaxLoopEq + k];
            C[j * kMaxLoopEq + k] = c;
        }
    }
    for (int j = 0; j < r; ++j) {
        double d = C[j * kMaxLoopEq + j];
        for (int k = 0; k < j; ++k) d -= C[j * kMaxLoopEq + k] * C[j * kMaxLoopEq + k];
        d = sqrt(d);
        C[j * kMaxLoopEq + j] = d;
        for (int i = j + 1; i < r; ++i) {
            double v = C[i * kMaxLoopEq + j];
            for (int k = 0; k < j; ++k) v -= C[i * kMaxLoopEq + k] * C[j * kMaxLoopEq + k];
            C[i * kMaxLoopEq + j] = v / d;
        }
    }
    for (int pass = 0; pass < 2; ++pass) {
        for (int i = 0; i < r; ++i) {
            double v = y[i];
            for (int k = 0; k < i; ++k) v -= C[i * kMaxLoopEq + k] * y[k];
            y[i] = v / C[i * kMaxLoopEq + i];
        }
        for (int i = r - 1; i >= 0; --i) {
            double v = y[i];
            for (int k = i + 1; k < r; ++k) v -= C[k * kMaxLoopEq + i] * y[k];
            y[i] = v / C[i * kMaxLoopEq + i];
        }
    }
    for (int i = 0; i < m; ++i) {
        double v = 0;
        for (int j = 0; j <= i && j < r; ++j) v += A[i * kMaxLoopEq + j] * y[j];
        b[F.piv[i]] = v;
    }
}

// Column j of G W G^T (kJacSweep) or G M^-1 G^T (kMInvSweep) for every j,
// three columns (one constraint) per sweep.
template <int NM, int KIND, class Wt>
__device__ __forceinline__ void loopGram(const LoopState& L, const Wt& wt, double* A) {
    const int nc = L.T.incons[L.inst];
    loopZeroAcc3(L);  // the accumulators of columns 1 and 2 held tree-pass values
    for (int c = 0; c < nc; ++c) {
        loopClearForces3(L);
        const LoopGeom Gc = loopGeom(L, c);
        for (int k = 0; k < 3; ++k) {
            V3d e = z3<double>();
            if (k == 0) e.x = 1.0; else if (k == 1) e.y = 1.0; else e.z = 1.0;
            loopAddForceK(L.S, Gc.s2, Gc.r2, e, k);
            loopAddForceK(L.S, Gc.s1, Gc.r1, -e, k);
        }
        loopSweep3<NM, KIND>(L, wt);
        for (int i = 0; i < nc; ++i) {
            const LoopGeom G = loopGeom(L, i);
            for (int k = 0; k < 3; ++k) {
                const V3d d = slotPoint(L.S, G.s2, slotB(k), G.r2) - slotPoint(L.S, G.s1, slotB(k), G.r1);
                A[(3 * i + 0) * kMaxLoopEq + 3 * c + k] = d.x;
                A[(3 * i + 1) * kMaxLoopEq + 3 * c + k] = d.y;
                A[(3 * i + 2) * kMaxLoopEq + 3 * c + k] = d.z;
            }
        }
    }
}

// loopGram with lane k < 3 of the group (gl, mask: the lane's index in the
// group and the group's lanes; absolute lane = the warp lane) sweeping
// column k of every constraint. A is filled on the group's first lane only;
// every lane of the group must call.
template <int NM, int KIND, class Wt>
__device__ __forceinline__ void loopGramLanes(const LoopState& L, const Wt& wt, double* A, int gl, unsigned mask) {
    const DevTables& T = L.T;
    const int nc = T.incons[L.inst];
    const int base = (int)(threadIdx.x & 31) - gl;
    const bool act = gl < 3;
    const int k = act ? gl : 0;
    if (act) {  // this column's accumulators held tree-pass values
        const int body0 = T.ibody[L.inst], nb = T.inb[L.inst];
        for (int lb = 0; lb < nb; ++lb) {
            const int row = body0 + lb;
            if ((T.info[row] & (F_MEMCHILD | F_LOOPPATH)) == (F_MEMCHILD | F_LOOPPATH)) {
                st3<double>(L.S, L.rec(row), recZaccK(k), z3<double>());
                st3<double>(L.S, L.rec(row), recZaccK(k) + 3, z3<double>());
            }
        }
    }
    for (int c = 0; c < nc; ++c) {
        if (act) {
            for (int c2 = 0; c2 < nc; ++c2) {
                int s1, s2;
                loopSlots(L, c2, s1, s2);
                if (s1 >= 0) { st3<double>(L.S, s1, slotF(k), z3<double>()); st3<double>(L.S, s1, slotF(k) + 3, z3<double>()); }
                if (s2 >= 0) { st3<double>(L.S, s2, slotF(k), z3<double>()); st3<double>(L.S, s2, slotF(k) + 3, z3<double>()); }
            }
            const LoopGeom Gc = loopGeom(L, c);
            V3d e = z3<double>();
            if (k == 0) e.x = 1.0; else if (k == 1) e.y = 1.0; else e.z = 1.0;
            loopAddForceK(L.S, Gc.s2, Gc.r2, e, k);
            loopAddForceK(L.S, Gc.s1, Gc.r1, -e, k);
            loopSweepColumn<NM, KIND>(L, wt, k);
        }
        for (int i = 0; i < nc; ++i) {
            V3d d = z3<double>();
            if (act) {
                const LoopGeom G = loopGeom(L, i);
                d = slotPoint(L.S, G.s2, slotB(k), G.r2) - slotPoint(L.S, G.s1, slotB(k), G.r1);
            }
            const double v[3] = {d.x, d.y, d.z};
#pragma unroll
            for (int r = 0; r < 3; ++r) {
                const double v1 = __shfl_sync(mask, v[r], base + 1), v2 = __shfl_sync(mask, v[r], base + 2);
                if (gl == 0) {
                    A[(3 * i + r) * kMaxLoopEq + 3 * c] = v[r];
                    A[(3 * i + r) * kMaxLoopEq + 3 * c + 1] = v1;
                    A[(3 * i + r) * kMaxLoopEq + 3 * c + 2] = v2;
                }
            }
        }
    }
}

// Loop forward dynamics after the tree RHS (which left the tree udot in out
// and A_GB in the slots). Returns SBG_INST_* bits. With DEFER_OUT the
// outward half of the final correction (udot -= M^-1 G^T lambda, every body)
// is left to loopCorrectionOutRows, which the lanes of a group run level by
// level.
template <int NM, bool DEFER_OUT = false, class Out>
__device__ __noinline__ int loopForwardDynamics(const LoopState& L, Out& out) {
    const DevTables& T = L.T;
    const int inst = L.inst;
    const SC64& S = L.S;
    const int nc = T.incons[inst], m = 3 * nc;
    loopZeroAcc(L);
    double lam[kMaxLoopEq];
    for (int c = 0; c < nc; ++c) {
        const LoopGeom G = loopGeom(L, c);
        const V3d aS = slotPoint(S, G.s2, kSlotA, G.r2) + slotCentripetal(S, G.s2, G.r2);
        const V3d aC = slotPoint(S, G.s1, kSlotA, G.r1) + slotCentripetal(S, G.s1, G.r1);
        const V3d d = aS - aC;
        lam[3 * c] = d.x; lam[3 * c + 1] = d.y; lam[3 * c + 2] = d.z;
    }
    double A[kMaxLoopEq * kMaxLoopEq];
    const NoWeights one{};
    loopGram<NM, kMInvSweep>(L, one, A);
    LoopFactor F;
    if (!loopCholFactor(m, A, kAccRelTol(m), F)) return SBG_INST_CHOLESKY_FAIL;
    loopCholSolve(m, A, F, lam);
    loopClearForces(L);
    for (int c = 0; c < nc; ++c) loopAddConstraintForce(L, loopGeom(L, c), mk3(lam[3 * c], lam[3 * c + 1], lam[3 * c + 2]));
    if constexpr (DEFER_OUT) {
        loopSweepIn<NM, kMInvSweep>(L, one);
    } else {
        loopSweep<NM, kMInvSweep, true>(L, one, [&](int row, int n, const double* ud) {
            const int uo = T.uoff[row];
            for (int i = 0; i < n; ++i) out.udot(uo + i, out.udotGet(uo + i) - ud[i]);
        });
    }
    return 0;
}

// loopForwardDynamics<NM, true> on a group of at least three lanes, the Gram
// columns spread over lanes 0-2 (loopGramLanes); the rest runs on the first
// lane as before, with the same results bit for bit. Every lane of the group
// calls; the status is the first lane's.
template <int NM, class Out>
__device__ __noinline__ int loopForwardDynamicsLanes(const LoopState& L, Out& out, int gl, unsigned mask) {
    const DevTables& T = L.T;
    const int inst = L.inst;
    const SC64& S = L.S;
    const int nc = T.incons[inst], m = 3 * nc;
    double lam[kMaxLoopEq];
    if (gl == 0) {
        loopZeroAcc(L);
        for (int c = 0; c < nc; ++c) {
            const LoopGeom G = loopGeom(L, c);
            const V3d aS = slotPoint(S, G.s2, kSlotA, G.r2) + slotCentripetal(S, G.s2, G.r2);
            const V3d aC = slotPoint(S, G.s1, kSlotA, G.r1) + slotCentripetal(S, G.s1, G.r1);
            const V3d d = aS - aC;
            lam[3 * c] = d.x; lam[3 * c + 1] = d.y; lam[3 * c + 2] = d.z;
        }
    }
    __syncwarp(mask);
    double A[kMaxLoopEq * kMaxLoopEq];
    const NoWeights one{};
    loopGramLanes<NM, kMInvSweep>(L, one, A, gl, mask);
    if (gl != 0) return 0;
    LoopFactor F;
    if (!loopCholFactor(m, A, kAccRelTol(m), F)) return SBG_INST_CHOLESKY_FAIL;
    loopCholSolve(m, A, F, lam);
    loopClearForces(L);
    for (int c = 0; c < nc; ++c) loopAddConstraintForce(L, loopGeom(L, c), mk3(lam[3 * c], lam[3 * c + 1], lam[3 * c + 2]));
    loopSweepIn<NM, kMInvSweep>(L, one);
    return 0;
}

// The outward half of the constraint-force correction on the lanes of a
// group (level-parallel layout): the same per-body step as the serial sweep,
// a level at a time, parents' accelerations through their records.
template <int NM, class Out>
__device__ __forceinline__ void loopCorrectionOutRows(const LoopState& L, Out& out, int gl, int G, unsigned mask) {
    const DevTables& T = L.T;
    const SC64& S = L.S;
    const int* ls = T.levStart + T.ilev[L.inst];
    const int nlev = T.inlev[L.inst];
    for (int lv = 0; lv < nlev; ++lv) {
        for (int lb = ls[lv] + gl; lb < ls[lv + 1]; lb += G) {
            const int row = L.body0 + lb;
            const int info = T.info[row];
            const int n = (info >> 4) & 15;
            const int parent = T.parent[row];  // local row = record of the parent
            const bool hp = parent >= 0;
            V3d pw = z3<double>(), pv = z3<double>();
            if (hp) {
                pw = ld3<double>(S, parent, 0);
                pv = ld3<double>(S, parent, 3);
            }
            double ud[6];
            const bool onPath = (info & F_LOOPPATH) != 0;
            if (n == 6) loopOut6<kMInvSweep>(L, lb, hp, onPath, pw, pv, ud);
            else loopOut<NM, kMInvSweep>(L, lb, n, hp, onPath, pw, pv, ud);
            const int uo = T.uoff[row];
            for (int i = 0; i < n; ++i) out.udot(uo + i, out.udotGet(uo + i) - ud[i]);
            st3<double>(S, lb, 0, pw);
            st3<double>(S, lb, 3, pv);
        }
        __syncwarp(mask);
    }
}

// ----------------------------------------------------------- projections
__device__ __forceinline__ double loopRMS(const double* v, int m) {
    double s = 0;
    for (int i = 0; i < m; ++i) s += v[i] * v[i];
    return m ? sqrt(s / m) : 0.0;
}
__device__ __forceinline__ double loopPerr(const LoopState& L, double* perr) {
    const int nc = L.T.incons[L.inst];
    for (int c = 0; c < nc; ++c) {
        const LoopGeom G = loopGeom(L, c);
        const V3d d = G.pS - G.pP;
        perr[3 * c] = d.x; perr[3 * c + 1] = d.y; perr[3 * c + 2] = d.z;
    }
    return loopRMS(perr, 3 * nc);
}
__device__ __forceinline__ double loopVerr(const LoopState& L, double* verr) {
    const int nc = L.T.incons[L.inst];
    for (int c = 0; c < nc; ++c) {
        const LoopGeom G = loopGeom(L, c);
        const V3d d = slotPoint(L.S, G.s2, 12, G.r2) - slotPoint(L.S, G.s1, 12, G.r1);
        verr[3 * c] = d.x; verr[3 * c + 1] = d.y; verr[3 * c + 2] = d.z;
    }
    return loopRMS(verr, 3 * nc);
}
__device__ __forceinline__ double& yAt(const LoopState& L, int k) { return L.y[L.base + (int64_t)k * L.stride]; }
__device__ __forceinline__ double& saveAt(const LoopState& L, int k) { return L.save[L.base + (int64_t)k * L.stride]; }
__device__ __forceinline__ double& deltaAt(const LoopState& L, int k) { return L.delta[L.base + (int64_t)k * L.stride]; }

__device__ __forceinline__ void loopNormalizeQuats(const LoopState& L) {
    const DevTables& T = L.T;
    const int body0 = T.ibody[L.inst], nb = T.inb[L.inst];
    for (int lb = 0; lb < nb; ++lb) {
        const int row = body0 + lb;
        if (!(T.info[row] & F_QUAT)) continue;
        const int qo = T.qoff[row];
        const double q0 = yAt(L, qo), q1 = yAt(L, qo + 1), q2 = yAt(L, qo + 2), q3 = yAt(L, qo + 3);
        const double len = sqrt(q0 * q0 + q1 * q1 + q2 * q2 + q3 * q3);
        yAt(L, qo) = q0 / len; yAt(L, qo + 1) = q1 / len; yAt(L, qo + 2) = q2 / len; yAt(L, qo + 3) = q3 / len;
    }
}

// Projection weights applied to the n values g = ~H F of a row in the
// inward half of a kJacSweep (du = D ~G lambda).
//   PosWeights (projectQ): D = NInv NInv^T of the current q: 4|q|^2 on the
//     rotational mobilities of a quaternion joint (Rotation.h:742-748); for a
//     joint in body-fixed X-Y-Z angles the 3x3 block NInv NInv^T with
//     NInv = [x, Rx y, Rx Ry z] (RigidBodyNodeSpec_Ball.h:266-300); 1 elsewhere
//   VelWeights (projectU): E^2, E = max(|u|, 1) of the entry u (saved)
// The Gram of the forward dynamics (kMInvSweep) applies none (NoWeights,
// defined with the sweeps).
struct PosWeights {
    const LoopState* L;
    __device__ __forceinline__ void apply(int row, int n, double* g) const {
        const DevTables& T = L->T;
        const int info = T.info[row], type = info & 15;
        const int qo = T.qoff[row];
        if (info & F_QUAT) {
            const double q0 = yAt(*L, qo), q1 = yAt(*L, qo + 1), q2 = yAt(*L, qo + 2), q3 = yAt(*L, qo + 3);
            const double w = 4 * (q0 * q0 + q1 * q1 + q2 * q2 + q3 * q3);
            for (int j = 0; j < 3 && j < n; ++j) g[j] = g[j] * w;
        } else if (type == T_BALL || type == T_FREE) {
            double s0, c0, s1, c1;
            sincos(yAt(*L, qo), &s0, &c0);
            sincos(yAt(*L, qo + 1), &s1, &c1);
            const double N[9] = {1, 0, s1, 0, c0, -s0 * c1, 0, s0, c0 * c1};
            double B[9];
            for (int r = 0; r < 3; ++r)
                for (int c = 0; c < 3; ++c)
                    B[3 * r + c] = N[3 * r] * N[3 * c] + N[3 * r + 1] * N[3 * c + 1] + N[3 * r + 2] * N[3 * c + 2];
            const double a0 = g[0], a1 = g[1], a2 = g[2];
            for (int r = 0; r < 3; ++r) g[r] = B[3 * r] * a0 + B[3 * r + 1] * a1 + B[3 * r + 2] * a2;
        }
    }
};
struct VelWeights {
    const LoopState* L;
    int nq;
    __device__ __forceinline__ void apply(int row, int n, double* g) const {
        const int uo = L->T.uoff[row];
        for (int j = 0; j < n; ++j) {
            const double a = fabs(saveAt(*L, nq + uo + j));
            const double e = a > 1 ? a : 1.0;
            g[j] = g[j] * (e * e);
        }
    }
};

// q -= N(q) du for one row's du (the unnormalized N of a quaternion,
// Rotation.h:712-719; N_P of body-fixed X-Y-Z angles, Rotation.h:395-406,
// the last q slot unused; the identity otherwise). Records du in delta.
__device__ __forceinline__ void loopStepQ(const LoopState& L, int row, int n, const double* du) {
    const DevTables& T = L.T;
    const int info = T.info[row], type = info & 15, qo = T.qoff[row];
    double dq[7];
    int nqb = n;
    if (info & F_QUAT) {
        const double e0 = yAt(L, qo) / 2, e1 = yAt(L, qo + 1) / 2, e2 = yAt(L, qo + 2) / 2, e3 = yAt(L, qo + 3) / 2;
        dq[0] = -e1 * du[0] - e2 * du[1] - e3 * du[2];
        dq[1] = e0 * du[0] + e3 * du[1] - e2 * du[2];
        dq[2] = -e3 * du[0] + e0 * du[1] + e1 * du[2];
        dq[3] = e2 * du[0] - e1 * du[1] + e0 * du[2];
        nqb = 4;
        if (type == T_FREE) { dq[4] = du[3]; dq[5] = du[4]; dq[6] = du[5]; nqb = 7; }
    } else if (type == T_BALL || type == T_FREE) {
        double s0, c0, s1, c1;
        sincos(yAt(L, qo), &s0, &c0);
        sincos(yAt(L, qo + 1), &s1, &c1);
        const double t = (s0 * du[1] - c0 * du[2]) * (1.0 / c1);
        dq[0] = du[0] + t * s1;
        dq[1] = c0 * du[1] + s0 * du[2];
        dq[2] = -t;
        if (type == T_FREE) { dq[3] = du[3]; dq[4] = du[4]; dq[5] = du[5]; dq[6] = 0; nqb = 7; }
        else { dq[3] = 0; nqb = 4; }
    } else {
        for (int j = 0; j < n; ++j) dq[j] = du[j];
    }
    for (int j = 0; j < nqb; ++j) {
        deltaAt(L, qo + j) = dq[j];
        yAt(L, qo + j) -= dq[j];
    }
}

__device__ __forceinline__ double loopTryFor(double tol) { return fmax(0.1 * tol, pow(2.220446049250313e-16, 0.875)); }

// Position projection (Newton); kinematics must be current for y. Leaves
// them current for the resulting y.
template <int NM>
__device__ __noinline__ bool loopProjectQ(const LoopState& L, double tol, bool localOnly) {
    const DevTables& T = L.T;
    const int nq = T.inq[L.inst], m = 3 * T.incons[L.inst];
    const int body0 = T.ibody[L.inst], nb = T.inb[L.inst];
    double perr[kMaxLoopEq], A[kMaxLoopEq * kMaxLoopEq];
    const double normOnEntry = loopPerr(L, perr);
    for (int k = 0; k < nq; ++k) {
        saveAt(L, k) = yAt(L, k);
        deltaAt(L, k) = 0.0;  // rows off the loop paths never move
    }
    const double tryFor = loopTryFor(tol);
    double achieved = normOnEntry, prev = normOnEntry;
    int its = 0;
    const PosWeights wq{&L};  // D = NInv NInv^T of the current q
    do {
        loopGram<NM, kJacSweep>(L, wq, A);
        LoopFactor F;
        if (!loopCholFactor(m, A, kProjRelTol(m), F)) return false;
        loopCholSolve(m, A, F, perr);
        loopClearForces(L);
        for (int c = 0; c < m / 3; ++c)
            loopAddConstraintForce(L, loopGeom(L, c), mk3(perr[3 * c], perr[3 * c + 1], perr[3 * c + 2]));
        // q -= N(q) du (loopStepQ)
        loopSweep<NM, kJacSweep>(L, wq, [&](int row, int n, const double* du) { loopStepQ(L, row, n, du); });
        loopKinematics<NM>(L);
        achieved = loopPerr(L, perr);
        ++its;
        if (localOnly && its >= 2 && achieved > prev) {
            for (int k = 0; k < nq; ++k) yAt(L, k) += deltaAt(L, k);
            loopKinematics<NM>(L);
            achieved = loopPerr(L, perr);
            break;
        }
        prev = achieved;
    } while (achieved > tryFor && its < 20);
    (void)body0; (void)nb;
    if (achieved > tol) {
        if (achieved >= normOnEntry) {
            for (int k = 0; k < nq; ++k) yAt(L, k) = saveAt(L, k);
            loopKinematics<NM>(L);
        }
        return false;
    }
    loopNormalizeQuats(L);
    loopKinematics<NM>(L);
    return true;
}

// Velocity projection at the current (q, u); recomputes the kinematics first.
template <int NM>
__device__ __noinline__ bool loopProjectU(const LoopState& L, double tol, bool force, double limit, bool localOnly) {
    const DevTables& T = L.T;
    const int nq = T.inq[L.inst], nu = T.inu[L.inst], m = 3 * T.incons[L.inst];
    loopKinematics<NM>(L);
    double verr[kMaxLoopEq], A[kMaxLoopEq * kMaxLoopEq];
    const double normOnEntry = loopVerr(L, verr);
    if (normOnEntry > limit) return false;
    if (normOnEntry == 0 || (normOnEntry <= tol && !force)) return true;
    for (int k = 0; k < nu; ++k) {
        saveAt(L, nq + k) = yAt(L, nq + k);
        deltaAt(L, nq + k) = 0.0;  // rows off the loop paths never move
    }
    // E^2 with E = max(|u|, 1) frozen at entry
    const VelWeights wu{&L, nq};
    loopGram<NM, kJacSweep>(L, wu, A);
    LoopFactor F;
    if (!loopCholFactor(m, A, kProjRelTol(m), F)) return false;
    const double tryFor = loopTryFor(tol);
    double achieved = normOnEntry, prev = normOnEntry;
    int its = 0;
    do {
        loopCholSolve(m, A, F, verr);
        loopClearForces(L);
        for (int c = 0; c < m / 3; ++c)
            loopAddConstraintForce(L, loopGeom(L, c), mk3(verr[3 * c], verr[3 * c + 1], verr[3 * c + 2]));
        loopSweep<NM, kJacSweep>(L, wu, [&](int row, int n, const double* du) {
            const int uo = nq + T.uoff[row];
            for (int j = 0; j < n; ++j) {
                deltaAt(L, uo + j) = du[j];
                yAt(L, uo + j) -= du[j];
            }
        });
        loopKinematics<NM>(L);
        achieved = loopVerr(L, verr);
        ++its;
        if (localOnly && its >= 2 && achieved > prev) {
            for (int k = 0; k < nu; ++k) yAt(L, nq + k) += deltaAt(L, nq + k);
            loopKinematics<NM>(L);
            achieved = loopVerr(L, verr);
            break;
        }
        prev = achieved;
    } while (achieved > tryFor && its < 7);
    if (achieved > tol) {
        if (achieved >= normOnEntry)
            for (int k = 0; k < nu; ++k) yAt(L, nq + k) = saveAt(L, nq + k);
        return false;
    }
    return true;
}

// ------------------------------- projections with the Gram over the lanes
// loopProjectQ / loopProjectU / loopProjectStep for a group of at least three
// lanes: the Gram (loopGramLanes) on lanes 0-2, everything else on the first
// lane, whose decisions (norms, failures) every lane takes by shuffle so that
// all of them run the same iterations. Same results bit for bit.
__device__ __forceinline__ double laneBcast(double v, int base, unsigned mask) { return __shfl_sync(mask, v, base); }
__device__ __forceinline__ int laneBcast(int v, int base, unsigned mask) { return __shfl_sync(mask, v, base); }

template <int NM>
__device__ __noinline__ bool loopProjectQLanes(const LoopState& L, double tol, bool localOnly, int gl, unsigned mask) {
    const DevTables& T = L.T;
    const int nq = T.inq[L.inst], m = 3 * T.incons[L.inst];
    const int base = (int)(threadIdx.x & 31) - gl;
    const bool lead = gl == 0;
    double perr[kMaxLoopEq], A[kMaxLoopEq * kMaxLoopEq];
    double normOnEntry = 0;
    if (lead) {
        normOnEntry = loopPerr(L, perr);
        for (int k = 0; k < nq; ++k) {
            saveAt(L, k) = yAt(L, k);
            deltaAt(L, k) = 0.0;  // rows off the loop paths never move
        }
    }
    normOnEntry = laneBcast(normOnEntry, base, mask);
    const double tryFor = loopTryFor(tol);
    double achieved = normOnEntry, prev = normOnEntry;
    int its = 0;
    const PosWeights wq{&L};  // D = NInv NInv^T of the current q
    do {
        __syncwarp(mask);  // the first lane's q and kinematics, before the Gram reads them
        loopGramLanes<NM, kJacSweep>(L, wq, A, gl, mask);
        int fail = 0;
        if (lead) {
            LoopFactor F;
            if (!loopCholFactor(m, A, kProjRelTol(m), F)) {
                fail = 1;
            } else {
                loopCholSolve(m, A, F, perr);
                loopClearForces(L);
                for (int c = 0; c < m / 3; ++c)
                    loopAddConstraintForce(L, loopGeom(L, c), mk3(perr[3 * c], perr[3 * c + 1], perr[3 * c + 2]));
                loopSweep<NM, kJacSweep>(L, wq, [&](int row, int n, const double* du) { loopStepQ(L, row, n, du); });
                loopKinematics<NM>(L);
                achieved = loopPerr(L, perr);
            }
        }
        if (laneBcast(fail, base, mask)) return false;
        achieved = laneBcast(achieved, base, mask);
        ++its;
        if (localOnly && its >= 2 && achieved > prev) {
            if (lead) {
                for (int k = 0; k < nq; ++k) yAt(L, k) += deltaAt(L, k);
                loopKinematics<NM>(L);
                achieved = loopPerr(L, perr);
            }
            achieved = laneBcast(achieved, base, mask);
            break;
        }
        prev = achieved;
    } while (achieved > tryFor && its < 20);
    if (achieved > tol) {
        if (lead && achieved >= normOnEntry) {
            for (int k = 0; k < nq; ++k) yAt(L, k) = saveAt(L, k);
            loopKinematics<NM>(L);
        }
        return false;
    }
    if (lead) {
        loopNormalizeQuats(L);
        loopKinematics<NM>(L);
    }
    return true;
}

template <int NM>
__device__ __noinline__ bool loopProjectULanes(const LoopState& L, double tol, bool force, double limit, bool localOnly,
                                               int gl, unsigned mask) {
    const DevTables& T = L.T;
    const int nq = T.inq[L.inst], nu = T.inu[L.inst], m = 3 * T.incons[L.inst];
    const int base = (int)(threadIdx.x & 31) - gl;
    const bool lead = gl == 0;
    double verr[kMaxLoopEq], A[kMaxLoopEq * kMaxLoopEq];
    double normOnEntry = 0;
    if (lead) {
        loopKinematics<NM>(L);
        normOnEntry = loopVerr(L, verr);
    }
    normOnEntry = laneBcast(normOnEntry, base, mask);
    if (normOnEntry > limit) return false;
    if (normOnEntry == 0 || (normOnEntry <= tol && !force)) return true;
    if (lead)
        for (int k = 0; k < nu; ++k) {
            saveAt(L, nq + k) = yAt(L, nq + k);
            deltaAt(L, nq + k) = 0.0;  // rows off the loop paths never move
        }
    __syncwarp(mask);  // the saved u, before the Gram's weights read it
    const VelWeights wu{&L, nq};
    loopGramLanes<NM, kJacSweep>(L, wu, A, gl, mask);
    LoopFactor F;
    int fail = lead ? (loopCholFactor(m, A, kProjRelTol(m), F) ? 0 : 1) : 0;
    if (laneBcast(fail, base, mask)) return false;
    const double tryFor = loopTryFor(tol);
    double achieved = normOnEntry, prev = normOnEntry;
    int its = 0;
    do {
        if (lead) {
            loopCholSolve(m, A, F, verr);
            loopClearForces(L);
            for (int c = 0; c < m / 3; ++c)
                loopAddConstraintForce(L, loopGeom(L, c), mk3(verr[3 * c], verr[3 * c + 1], verr[3 * c + 2]));
            loopSweep<NM, kJacSweep>(L, wu, [&](int row, int n, const double* du) {
                const int uo = nq + T.uoff[row];
                for (int j = 0; j < n; ++j) {
                    deltaAt(L, uo + j) = du[j];
                    yAt(L, uo + j) -= du[j];
                }
            });
            loopKinematics<NM>(L);
            achieved = loopVerr(L, verr);
        }
        achieved = laneBcast(achieved, base, mask);
        ++its;
        if (localOnly && its >= 2 && achieved > prev) {
            if (lead) {
                for (int k = 0; k < nu; ++k) yAt(L, nq + k) += deltaAt(L, nq + k);
                loopKinematics<NM>(L);
                achieved = loopVerr(L, verr);
            }
            achieved = laneBcast(achieved, base, mask);
            break;
        }
        prev = achieved;
    } while (achieved > tryFor && its < 7);
    if (achieved > tol) {
        if (lead && achieved >= normOnEntry)
            for (int k = 0; k < nu; ++k) yAt(L, nq + k) = saveAt(L, nq + k);
        return false;
    }
    return true;
}

template <int NM>
__device__ __noinline__ int loopProjectStepLanes(const LoopState& L, double quatNorm, double tol, double limit, bool force,
                                                 int gl, unsigned mask) {
    const int base = (int)(threadIdx.x & 31) - gl;
    const bool lead = gl == 0;
    double perr[kMaxLoopEq];
    double perrNorm = 0;
    if (lead) {
        loopZeroAcc(L);
        loopKinematics<NM>(L);
        perrNorm = loopPerr(L, perr);
    }
    perrNorm = laneBcast(perrNorm, base, mask);
    const double normOnEntry = fmax(perrNorm, quatNorm);
    bool ok = true;
    if (normOnEntry > limit) {
        ok = false;
    } else if (perrNorm == 0 || (perrNorm <= tol && !force)) {
        if (lead && (quatNorm > tol || force)) loopNormalizeQuats(L);
    } else {
        ok = loopProjectQLanes<NM>(L, tol, true, gl, mask);
    }
    __syncwarp(mask);
    if (ok) ok = loopProjectULanes<NM>(L, tol, force, limit, true, gl, mask);
    return ok ? 0 : SBG_INST_PROJECTION_FAILED;
}

// Integrator::initialize: ProjectOptions::ForceProjection, no projection
// limit, not LocalOnly (IntegratorRep.h:856-895). Returns SBG_INST_* bits.
template <int NM>
__device__ __noinline__ int loopInitialize(const LoopState& L, double tol) {
    double perr[kMaxLoopEq];
    loopZeroAcc(L);
    loopKinematics<NM>(L);
    bool ok = true;
    if (loopPerr(L, perr) == 0) loopNormalizeQuats(L);
    else ok = loopProjectQ<NM>(L, tol, false);
    if (!loopProjectU<NM>(L, tol, true, INFINITY, false)) ok = false;
    return ok ? 0 : SBG_INST_PROJECTION_FAILED;
}

// After an accepted step whose error passed the gate of
// AbstractIntegratorRep.cpp:158-166: projectQ then projectU (:168-205),
// both LocalOnly, with the projection limit. Returns SBG_INST_* bits.
template <int NM>
__device__ __noinline__ int loopProjectStep(const LoopState& L, double quatNorm, double tol, double limit, bool force) {
    double perr[kMaxLoopEq];
    loopZeroAcc(L);
    loopKinematics<NM>(L);
    const double perrNorm = loopPerr(L, perr);
    const double normOnEntry = fmax(perrNorm, quatNorm);
    bool ok = true;
    if (normOnEntry > limit) {
        ok = false;
    } else if (perrNorm == 0 || (perrNorm <= tol && !force)) {
        if (quatNorm > tol || force) loopNormalizeQuats(L);
    } else {
        ok = loopProjectQ<NM>(L, tol, true);
    }
    if (ok) ok = loopProjectU<NM>(L, tol, force, limit, true);
    return ok ? 0 : SBG_INST_PROJECTION_FAILED;
}
