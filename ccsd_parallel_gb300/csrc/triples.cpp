// CCSDT-1a on the CCSD engine (the reference's CCSDT::Calc_Energy(toler, 1),
// ccsdt.cpp:255-271): every update forms T1/T2 from the previous T3 and T3
// from the previous T2, in the reference's spin-orbital form (spin orbital
// P = 2p + spin, O = 2 nocc, V = 2 nvir).  The closed-shell numerators are
// the alpha-beta blocks of the spin-orbital ones: R1[i][a] += R1so(2a, 2i),
// R[i][j][a][b] += R2so(2a, 2b+1, 2i, 2j+1).
#include "engine.h"

namespace ccsd {

namespace {
inline MatView mv(const double *p, Dim r, Dim c) {
    MatView m;
    m.p = p;
    m.row = r;
    m.col = c;
    return m;
}
inline OutView ovw(double *p, Dim r, Dim c) {
    OutView m;
    m.p = p;
    m.row = r;
    m.col = c;
    return m;
}
}  // namespace

void Engine::triples_setup() {
    const size_t O = 2 * (size_t)o_, V = 2 * (size_t)v_;
    const size_t n3 = V * V * V * O * O * O;
    t3_.ensure(n3);
    y3_.ensure(n3);
    z3_.ensure(n3);
    t2so_.ensure(V * V * O * O);
    so_vvvo_.ensure(V * V * V * O);
    so_ovoo_.ensure(O * V * O * O);
    so_oovv_.ensure(O * O * V * V);
    so_vovv_.ensure(V * O * V * V);
    so_ooov_.ensure(O * O * O * V);
    DBuf *blocks[5] = {&so_vvvo_, &so_ovoo_, &so_oovv_, &so_vovv_, &so_ooov_};
    for (int kind = 0; kind < 5; ++kind)
        k_so_block(kind, o_, v_, ovov_.p, ovoo_.p, ovvv_.p, nullptr, nullptr, nullptr, blocks[kind]->p, st_);
    if (opt_.method >= CCSD_METHOD_CCSDT3) {
        if (wv_.n < (size_t)v_ * v_ * v_ * v_)
            throw Error(CCSD_ERR_INVALID_ARG, "CCSDT-3 needs (ac|bd): set method CCSD_METHOD_CCSDT3 at ccsd_create");
        so_voov_.ensure(V * O * O * V);
        so_oooo_.ensure(O * O * O * O);
        so_vvvv_.ensure(V * V * V * V);
        k_so_block(5, o_, v_, ovov_.p, ovoo_.p, ovvv_.p, oovv_.p, oooo_.p, wv_.p, so_voov_.p, st_);
        k_so_block(6, o_, v_, ovov_.p, ovoo_.p, ovvv_.p, oovv_.p, oooo_.p, wv_.p, so_oooo_.p, st_);
        k_so_block(7, o_, v_, ovov_.p, ovoo_.p, ovvv_.p, oovv_.p, oooo_.p, wv_.p, so_vvvv_.p, st_);
        tauso_.ensure(V * V * O * O);
        for (DBuf *b : {&p1_, &p2_, &p4_, &d14_, &e15_}) b->ensure(V * O * O * V);
        p3_.ensure(O * O * O * O);
        g15_.ensure(O * O * O * O);
        a1_.ensure(O * O * O * V);
        x14_.ensure(V * V * O * V);
        x15_.ensure(V * O * O * O);
    }
    if (opt_.method >= CCSD_METHOD_CCSDT) {
        x3_.ensure(O * O * O * O);
        x4_.ensure(V * V * V * V);
        x6_.ensure(V * O * O * V);
        x7_.ensure(O * O);
        x8_.ensure(V * V);
        fsoT_.ensure(V * O);
    }
    t3_.zero(st_);  // T3 starts at zero (the first update is CCSD-like)
    y3_.zero(st_);  // spin-forbidden blocks of Y and Z are never written
    z3_.zero(st_);
    if (opt_.method >= CCSD_METHOD_CCSDT2) {
        x1d_.ensure(V * V * V * O);
        x2d_.ensure(O * V * O * O);
        x12_.ensure(V * V * O * V);
        x13_.ensure(V * O * O * O);
        q12_.ensure(n3);
        q13_.ensure(n3);
        q12_.zero(st_);  // spin-forbidden blocks are never written
        q13_.zero(st_);
    }
    if (opt_.method >= CCSD_METHOD_CCSDT1B) {
        const size_t o = o_, v = v_;
        t1so_.ensure(V * O);
        g1b_.ensure(v * o * o * o);
        g2b_.ensure(v * o * o * o);
        h3b_.ensure(v * v * o * v);
        h4b_.ensure(v * v * o * v);
        f1b_.ensure(O * V);
        w5b_.ensure(v * v * O * O);
    }
}

// CCSDT-1b (ccsdt.cpp:676-700): R2 += 1/2 sum_{c,d,k,l} <kl||cd> [- t3(acd,ikj) t1(b,l)
//   + t3(bcd,ikj) t1(a,l) - t3(adb,klj) t1(c,i) + t3(adb,kli) t1(c,j) + 2 t3(abc,ijk) t1(d,l)]
// from the previous t3 and t1, in the alpha-beta block (a = 2a', b = 2b'+1, i = 2i',
// j = 2j'+1), where t1(b,l) fixes l = 2l'+1, t1(a,l) l = 2l', t1(c,i) c = 2c' and
// t1(c,j) c = 2c'+1.  Intermediates (spatial primed indices, the other spins summed
// over the spin-conserving blocks):
//   G1(a',i',j',l') = sum_{c,d,k} <k,2l'+1||c,d> t3[2a'][c][d][2i'][k][2j'+1]
//   G2(b',i',j',l') = sum_{c,d,k} <k,2l'||c,d>   t3[2b'+1][c][d][2i'][k][2j'+1]
//   H3(a',b',j',c') = sum_{d,k,l} <k,l||2c',d>   t3[2a'][d][2b'+1][k][l][2j'+1]
//   H4(a',b',i',c') = sum_{d,k,l} <k,l||2c'+1,d> t3[2a'][d][2b'+1][k][l][2i']
//   f(k,c) = sum_{d,l} <kl||cd> t1(d,l),  W5[a'][b'][i][j] = sum_{c,k} t3[2a'][2b'+1][c][i][j][k] f(k,c)
void Engine::triples_1b_terms() {
    const int64_t o = o_, v = v_, O = 2 * o, V = 2 * v, O2 = O * O, O3 = O2 * O, VO3 = V * O3, V2O3 = V * VO3;
    const int io = (int)o, iv = (int)v;
    const uint32_t uo = (uint32_t)o, uv = (uint32_t)v;
    const double *t3 = t3_.p, *t1 = t1_.p, *g = so_oovv_.p;  // g = <kl||cd> at [k][l][c][d]
    const int64_t gk = O * V * V, gl = V * V, gc = V;
    struct Spins {
        int s0, s1, s2;
    };
    // G1: (sc, sd, sk) with sc + sd = sk + 1;  G2: sc + sd = sk
    const Spins s1[3] = {{0, 1, 0}, {1, 0, 0}, {1, 1, 1}};
    const Spins s2[3] = {{0, 0, 0}, {0, 1, 1}, {1, 0, 1}};
    const Dim rows_xij = ix3(uo, uo, 2 * V2O3, 2 * O2, 2);  // (x', i', j') of t3[x][.][.][i][.][j]
    const Dim K_cdk = ix3(uv, uo, 2 * VO3, 2 * O3, 2 * O);  // (c', d', k') in t3[.][c][d][.][k][.]
    const Dim Kg_cdk = ix3(uv, uo, 2 * gc, 2, 2 * gk);      // (c', d', k') in <kl||cd>
    const Dim rows_G = ix3(uo, uo, o * o * o, o * o, o);     // G[x'][i'][j'][l']
    for (int q = 0; q < 3; ++q) {
        const Spins &p = s1[q], &r = s2[q];
        gemm(iv * io * io, io, (int)(v * v * o), 1.0, mv(t3 + p.s0 * VO3 + p.s1 * O3 + p.s2 * O + 1, rows_xij, K_cdk),
             mv(g + p.s2 * gk + gl + p.s0 * gc + p.s1, ix1(2 * gl), Kg_cdk), q ? 1.0 : 0.0,
             ovw(g1b_.p, rows_G, ix1(1)), 0, 420 + q, "T3T1_G1");
        gemm(iv * io * io, io, (int)(v * v * o), 1.0,
             mv(t3 + V2O3 + r.s0 * VO3 + r.s1 * O3 + r.s2 * O + 1, rows_xij, K_cdk),
             mv(g + r.s2 * gk + r.s0 * gc + r.s1, ix1(2 * gl), Kg_cdk), q ? 1.0 : 0.0, ovw(g2b_.p, rows_G, ix1(1)),
             0, 423 + q, "T3T1_G2");
    }
    // R[i'][j'][a'][b'] += -1/2 sum_l' G1(a',i',j',l') t1[l'][b'] + 1/2 sum_l' G2(b',i',j',l') t1[l'][a']
    const Dim G_ijx = ix3(uo, uv, o * o, o, o * o * o);  // rows (i', j', x') of G
    gemm(io * io * iv, iv, io, -0.5, mv(g1b_.p, G_ijx, ix1(1)), mv(t1, ix1(1), ix1(v)), 1.0,
         ovw(R_.p, ix3(uo, uv, o * v * v, v * v, v), ix1(1)), 0, 0, "T3T1_G1t1");
    gemm(io * io * iv, iv, io, 0.5, mv(g2b_.p, G_ijx, ix1(1)), mv(t1, ix1(1), ix1(v)), 1.0,
         ovw(R_.p, ix3(uo, uv, o * v * v, v * v, 1), ix1(v)), 0, 0, "T3T1_G2t1");

    // H3: (sd, sk, sl) with sd = sk + sl;  H4: sk + sl = sd + 1
    const Spins s3[3] = {{0, 0, 0}, {1, 0, 1}, {1, 1, 0}};
    const Spins s4[3] = {{0, 0, 1}, {0, 1, 0}, {1, 1, 1}};
    const Dim rows_abx = ix3(uv, uo, 2 * V2O3, 2 * O3, 2);   // (a', b', x') of t3[a][.][b][.][.][x]
    const Dim K_dkl = ix3(uo, uo, 2 * VO3, 2 * O2, 2 * O);   // (d', k', l') in t3[.][d][.][k][l][.]
    const Dim Kg_dkl = ix3(uo, uo, 2, 2 * gk, 2 * gl);       // (d', k', l') in <kl||cd>
    const Dim rows_H = ix3(uv, uo, v * o * v, o * v, v);     // H[a'][b'][x'][c']
    for (int q = 0; q < 3; ++q) {
        const Spins &p = s3[q], &r = s4[q];
        gemm(iv * iv * io, iv, (int)(v * o * o), 1.0,
             mv(t3 + p.s0 * VO3 + O3 + p.s1 * O2 + p.s2 * O + 1, rows_abx, K_dkl),
             mv(g + p.s1 * gk + p.s2 * gl + p.s0, ix1(2 * gc), Kg_dkl), q ? 1.0 : 0.0, ovw(h3b_.p, rows_H, ix1(1)), 0,
             426 + q, "T3T1_H3");
        gemm(iv * iv * io, iv, (int)(v * o * o), 1.0, mv(t3 + r.s0 * VO3 + O3 + r.s1 * O2 + r.s2 * O, rows_abx, K_dkl),
             mv(g + r.s1 * gk + r.s2 * gl + gc + r.s0, ix1(2 * gc), Kg_dkl), q ? 1.0 : 0.0,
             ovw(h4b_.p, rows_H, ix1(1)), 0, 429 + q, "T3T1_H4");
    }
    // R[i'][j'][a'][b'] += -1/2 sum_c' H3(a',b',j',c') t1[i'][c'] + 1/2 sum_c' H4(a',b',i',c') t1[j'][c']
    gemm(iv * iv * io, io, iv, -0.5, mv(h3b_.p, rows_H, ix1(1)), mv(t1, ix1(v), ix1(1)), 1.0,
         ovw(R_.p, ix3(uv, uo, v, 1, v * v), ix1(o * v * v)), 0, 0, "T3T1_H3t1");
    gemm(iv * iv * io, io, iv, 0.5, mv(h4b_.p, rows_H, ix1(1)), mv(t1, ix1(v), ix1(1)), 1.0,
         ovw(R_.p, ix3(uv, uo, v, 1, o * v * v), ix1(v * v)), 0, 0, "T3T1_H4t1");

    // f(k,c) = sum_{l,d} <kl||cd> t1so[d][l]  (O x V; zero unless sk = sc)
    k_t1_spin(io, iv, t1, t1so_.p, st_);
    gemm((int)(O * V), 1, (int)(O * V), 1.0, mv(g, ix2((uint32_t)V, gk, gc), ix2((uint32_t)V, gl, 1)),
         mv(t1so_.p, ix1(0), ix2((uint32_t)V, 1, O)), 0.0, ovw(f1b_.p, ix1(1), ix1(0)), 0, 0, "T3T1_f");
    // W5[a'][b'][i][j] = sum_{c,k} t3[2a'][2b'+1][c][i][j][k] f(k,c), rows (a', b', i O + j)
    gemm((int)(v * v * O2), 1, (int)(V * O), 1.0,
         mv(t3 + VO3, ix3(uv, (uint32_t)O2, 2 * V2O3, 2 * VO3, O), ix2((uint32_t)O, O3, 1)),
         mv(f1b_.p, ix1(0), ix2((uint32_t)O, 1, V)), 0.0, ovw(w5b_.p, ix1(1), ix1(0)), 0, 0, "T3T1_ft3");
    // R[i'][j'][a'][b'] += W5[a'][b'][2i'][2j'+1]  (1/2 x 2)
    axpby(io * io * iv, iv, 1.0, mv(w5b_.p + 1, ix3(uo, uv, 2 * O, 2, v * O2), ix1(O2)), 1.0,
          ovw(R_.p, ix3(uo, uv, o * v * v, v * v, v), ix1(1)));
}

// CCSDT-2 (ccsdt.cpp:1078-1130, 2301-2390): from this T2,
//   X12[a][b][i][d] = sum_{l,e} <lb||ed> t2so[a][e][i][l]    (<lb||ed> = -<bl||ed>)
//   X13[a][l][i][j] = -sum_{m,d} <ml||dj> t2so[a][d][i][m]   (<ml||dj> = -<ml||jd>)
//   Q12[a][b][c][i][j][k] = sum_e X12[a][b][i][e] t2so[e][c][j][k]
//   Q13[a][b][c][i][j][k] = sum_m X13[a][m][i][j] t2so[b][c][m][k]
// Q12 and Q13 conserve spin like Y and Z: 18 spin blocks each, as stride-2 views.
void Engine::triples_m3_products() {
    const int64_t o = o_, v = v_, O = 2 * o, V = 2 * v, O2 = O * O, O3 = O2 * O, VO3 = V * O3, V2O3 = V * VO3;
    const uint32_t uo = (uint32_t)o, uv = (uint32_t)v;
    const int64_t VO2 = V * O2;
    // X12: M = (a,i), N = (b,d), K = (l,e)
    gemm((int)(V * O), (int)(V * V), (int)(O * V), -1.0,
         mv(t2so_.p, ix2((uint32_t)O, VO2, O), ix2((uint32_t)V, 1, O2)),
         mv(so_vovv_.p, ix2((uint32_t)V, O * V * V, 1), ix2((uint32_t)V, V * V, V)), 0.0,
         ovw(x12_.p, ix2((uint32_t)O, V * O * V, V), ix2((uint32_t)V, O * V, 1)), 0, 0, "T3_X12");
    // X13: M = (a,i), N = (l,j), K = (m,d)
    gemm((int)(V * O), (int)O2, (int)(O * V), 1.0,
         mv(t2so_.p, ix2((uint32_t)O, VO2, O), ix2((uint32_t)V, 1, O2)),
         mv(so_ooov_.p, ix2((uint32_t)O, O * V, V), ix2((uint32_t)V, O2 * V, 1)), 0.0,
         ovw(x13_.p, ix2((uint32_t)O, O3, O), ix2((uint32_t)O, O2, 1)), 0, 0, "T3_X13");
    if (opt_.method >= CCSD_METHOD_CCSDT3) triples_m4_terms();  // T1 terms of X12/X13, X14/X15 into Z/Y
    const int64_t X12a = V * O * V, X12b = O * V, X12i = V;  // X12[a][b][i][d] strides
    for (int sa = 0; sa < 2; ++sa)
        for (int sb = 0; sb < 2; ++sb)
            for (int si = 0; si < 2; ++si) {
                // Q12: se = sa + sb - si, (sc, sj, sk) with se + sc = sj + sk;  M = (a,b,i), N = (c,j,k), K = e
                const int se = sa + sb - si;
                if (se < 0 || se > 1) continue;
                const MatView Av = mv(x12_.p + sa * X12a + sb * X12b + si * X12i + se,
                                      ix3(uv, uo, 2 * X12a, 2 * X12b, 2 * X12i), ix1(2));
                for (int sj = 0; sj < 2; ++sj)
                    for (int sk = 0; sk < 2; ++sk) {
                        const int sc = sj + sk - se;
                        if (sc < 0 || sc > 1) continue;
                        const double *B = t2so_.p + se * VO2 + sc * O2 + sj * O + sk;
                        double *Cp = q12_.p + sa * V2O3 + sb * VO3 + si * O2 + sc * O3 + sj * O + sk;
                        gemm((int)(v * v * o), (int)(v * o * o), (int)v, 1.0, Av,
                             mv(B, ix3(uo, uo, 2 * O2, 2 * O, 2), ix1(2 * VO2)), 0.0,
                             ovw(Cp, ix3(uv, uo, 2 * V2O3, 2 * VO3, 2 * O2), ix3(uo, uo, 2 * O3, 2 * O, 2)),
                             -(500 + sa * 4 + sb * 2 + si), -(510 + se * 8 + sc * 4 + sj * 2 + sk), "T3_Q12");
                    }
            }
    for (int sa = 0; sa < 2; ++sa)
        for (int si = 0; si < 2; ++si)
            for (int sj = 0; sj < 2; ++sj) {
                // Q13: sm = si + sj - sa, (sb, sc, sk) with sb + sc = sm + sk;  M = (a,i,j), N = (b,c,k), K = m
                const int sm = si + sj - sa;
                if (sm < 0 || sm > 1) continue;
                const MatView Av = mv(x13_.p + sa * O3 + sm * O2 + si * O + sj, ix3(uo, uo, 2 * O3, 2 * O, 2),
                                      ix1(2 * O2));
                for (int sb = 0; sb < 2; ++sb)
                    for (int sc = 0; sc < 2; ++sc) {
                        const int sk = sb + sc - sm;
                        if (sk < 0 || sk > 1) continue;
                        const double *B = t2so_.p + sb * VO2 + sc * O2 + sm * O + sk;
                        double *Cp = q13_.p + sa * V2O3 + si * O2 + sj * O + sb * VO3 + sc * O3 + sk;
                        gemm((int)(v * o * o), (int)(v * v * o), (int)o, 1.0, Av,
                             mv(B, ix3(uv, uo, 2 * VO2, 2 * O2, 2), ix1(2 * O)), 0.0,
                             ovw(Cp, ix3(uo, uo, 2 * V2O3, 2 * O2, 2 * O), ix3(uv, uo, 2 * VO3, 2 * O3, 2)),
                             -(520 + sa * 4 + si * 2 + sj), -(530 + sm * 8 + sb * 4 + sc * 2 + sk), "T3_Q13");
                    }
            }
}

// CCSDT-3 (ccsdt.cpp:1028-1070, 2043-2125, 2321-2383), from this T1 and T2 (t1so, t2so):
//   X12[a][b][i][d] -= sum_l <al||id> t1[b][l] + sum_l t1[a][l] P1[l][b][i][d] + sum_m t1[b][m] P2[a][i][m][d]
//   X13[a][l][i][j] += sum_m t1[a][m] P3[m][l][i][j] - sum_e P2[a][i][l][e] t1[e][j] - sum_d <al||id> t1[d][j]
//     P1[l][b][i][d] = sum_e <lb||ed> t1[e][i]           (<lb||ed> = -<bl||ed>)
//     P2[a][i][m][d] = sum_{l,e} t2[a][e][i][l] <lm||ed>
//     P3[m][l][i][j] = sum_d <ml||dj> t1[d][i]           (<ml||dj> = -<ml||jd>)
//   X14[a][b][i][d] = sum_e <ab||ed> t1[e][i] + 1/2 sum_{l,m} t2[a][b][l][m] A1[l][m][i][d]
//                     - sum_m t2[a][b][i][m] f[m][d] + sum_{l,m} t1[a][l] t1[b][m] (A1 + <lm||id>)[l][m][i][d]
//     A1[l][m][i][d] = sum_e <lm||ed> t1[e][i],  f[m][d] = sum_{l,e} <ml||de> t1[e][l] (the CCSDT-1b f)
//   X15[a][l][i][j] = -sum_e E[a][l][i][e] t1[e][j] + sum_m t1[a][m] G[m][l][i][j]
//     E[a][l][i][e] = sum_d <al||de> t1[d][i],  G = <ml||ij> + 1/2 sum_{d,e} <ml||de> tau[d][e][i][j]
//   Z -= sum_e X14[a][b][i][e] t2[e][c][j][k]   (the antisymmetriser of X2's term, opposite sign)
//   Y += sum_m X15[a][m][i][j] t2[b][c][m][k]   (the antisymmetriser of X1's term)
void Engine::triples_m4_terms() {
    const int64_t o = o_, v = v_, O = 2 * o, V = 2 * v, O2 = O * O, O3 = O2 * O, VO3 = V * O3, V2O3 = V * VO3;
    const int64_t VO2 = V * O2, OV = O * V, VOV = V * O * V, O2V = O2 * V, V2 = V * V;
    const uint32_t uO = (uint32_t)O, uV = (uint32_t)V, uo = (uint32_t)o, uv = (uint32_t)v;
    const int iO = (int)O, iV = (int)V;
    const double *t1s = t1so_.p, *t2s = t2so_.p;
    const MatView t1_xl = mv(t1s, ix1(O), ix1(1));  // t1[x][l]: rows x, K l
    const MatView t1_ie = mv(t1s, ix1(1), ix1(O));  // t1[e][i]: rows i, K e
    const Dim rows_aid_x12 = ix3(uO, uV, VOV, V, 1);  // (a,i,d) of a [a][b][i][d] array
    // ---- X12
    gemm(iV * iO * iV, iV, iO, -1.0, mv(so_voov_.p, ix3(uO, uV, O2V, V, 1), ix1(OV)), t1_xl, 1.0,
         ovw(x12_.p, rows_aid_x12, ix1(OV)), 0, 0, "T3_X12_voov_t1");
    gemm(iO * iV * iV, iO, iV, -1.0, mv(so_vovv_.p, ix3(uV, uV, V2, O * V2, 1), ix1(V)), t1_ie, 0.0,
         ovw(p1_.p, ix3(uV, uV, VOV, OV, 1), ix1(V)), 0, 0, "T3_P1");
    gemm(iV * iO * iV, iV, iO, -1.0, mv(p1_.p, ix1(1), ix1(VOV)), t1_xl, 1.0, ovw(x12_.p, ix1(1), ix1(VOV)), 0, 0,
         "T3_X12_P1");
    gemm(iV * iO, iO * iV, iO * iV, 1.0, mv(t2s, ix2(uO, VO2, O), ix2(uV, 1, O2)),
         mv(so_oovv_.p, ix2(uV, V2, 1), ix2(uV, O * V2, V)), 0.0, ovw(p2_.p, ix2(uO, O2V, OV), ix1(1)), 0, 0, "T3_P2");
    gemm(iV * iO * iV, iV, iO, -1.0, mv(p2_.p, ix3(uO, uV, O2V, OV, 1), ix1(V)), t1_xl, 1.0,
         ovw(x12_.p, rows_aid_x12, ix1(OV)), 0, 0, "T3_X12_P2");
    // ---- X13
    gemm((int)O3, iO, iV, -1.0, mv(so_ooov_.p, ix1(V), ix1(1)), t1_ie, 0.0,
         ovw(p3_.p, ix3(uO, uO, O3, O2, 1), ix1(O)), 0, 0, "T3_P3");
    gemm((int)O3, iV, iO, 1.0, mv(p3_.p, ix1(1), ix1(O3)), t1_xl, 1.0, ovw(x13_.p, ix1(1), ix1(O3)), 0, 0,
         "T3_X13_P3");
    gemm(iV * iO * iO, iO, iV, -1.0, mv(p2_.p, ix3(uO, uO, O2V, V, OV), ix1(1)), t1_ie, 1.0,
         ovw(x13_.p, ix3(uO, uO, O3, O2, O), ix1(1)), 0, 0, "T3_X13_P2");
    gemm(iV * iO * iO, iO, iV, -1.0, mv(so_voov_.p, ix1(V), ix1(1)), t1_ie, 1.0, ovw(x13_.p, ix1(O), ix1(1)), 0, 0,
         "T3_X13_voov_t1");
    // ---- X14
    gemm(iV * iV * iV, iO, iV, 1.0, mv(so_vvvv_.p, ix2(uV, V2, 1), ix1(V)), t1_ie, 0.0,
         ovw(x14_.p, ix2(uV, OV, 1), ix1(V)), 0, 0, "T3_X14_vvvv_t1");
    gemm(iO * iO * iV, iO, iV, 1.0, mv(so_oovv_.p, ix2(uV, V2, 1), ix1(V)), t1_ie, 0.0,
         ovw(a1_.p, ix2(uV, OV, 1), ix1(V)), 0, 0, "T3_A1");
    gemm(iV * iV, iO * iV, (int)O2, 0.5, mv(t2s, ix1(O2), ix1(1)), mv(a1_.p, ix1(1), ix1(OV)), 1.0,
         ovw(x14_.p, ix1(OV), ix1(1)), 0, 0, "T3_X14_t2A1");
    gemm(iV * iV * iO, iV, iO, -1.0, mv(t2s, ix1(O), ix1(1)), mv(f1b_.p, ix1(1), ix1(V)), 1.0,
         ovw(x14_.p, ix1(V), ix1(1)), 0, 0, "T3_X14_t2f");
    axpby((int)O3, iV, 1.0, mv(so_ooov_.p, ix1(V), ix1(1)), 1.0, ovw(a1_.p, ix1(V), ix1(1)));  // A1 + <lm||id>
    gemm(iO * iO * iV, iV, iO, 1.0, mv(a1_.p, ix1(1), ix1(O2V)), t1_xl, 0.0, ovw(d14_.p, ix1(1), ix1(O2V)), 0, 0,
         "T3_D14");
    gemm(iV * iO * iV, iV, iO, 1.0, mv(d14_.p, ix3(uO, uV, O2V, V, 1), ix1(OV)), t1_xl, 1.0,
         ovw(x14_.p, rows_aid_x12, ix1(OV)), 0, 0, "T3_X14_t1t1");
    // ---- X15
    gemm(iV * iO * iV, iO, iV, 1.0, mv(so_vovv_.p, ix2(uV, V2, 1), ix1(V)), t1_ie, 0.0,
         ovw(e15_.p, ix2(uV, OV, 1), ix1(V)), 0, 0, "T3_E15");
    gemm(iV * iO * iO, iO, iV, -1.0, mv(e15_.p, ix1(V), ix1(1)), t1_ie, 0.0, ovw(x15_.p, ix1(O), ix1(1)), 0, 0,
         "T3_X15_E");
    k_tau_spin((int)o, (int)v, t2s, t1s, tauso_.p, st_);
    copy(g15_.p, so_oooo_.p, (size_t)(O2 * O2));
    gemm((int)O2, (int)O2, (int)V2, 0.5, mv(so_oovv_.p, ix1(V2), ix1(1)), mv(tauso_.p, ix1(1), ix1(O2)), 1.0,
         ovw(g15_.p, ix1(O2), ix1(1)), 0, 0, "T3_G15");
    gemm((int)O3, iV, iO, 1.0, mv(g15_.p, ix1(1), ix1(O3)), t1_xl, 1.0, ovw(x15_.p, ix1(1), ix1(O3)), 0, 0,
         "T3_X15_G");
    // ---- Q14 into Z, Q15 into Y (the spin blocks and t2 views of Q12 and Q13)
    for (int sa = 0; sa < 2; ++sa)
        for (int sb = 0; sb < 2; ++sb)
            for (int si = 0; si < 2; ++si) {
                const int se = sa + sb - si;
                if (se < 0 || se > 1) continue;
                const MatView Av =
                    mv(x14_.p + sa * VOV + sb * OV + si * V + se, ix3(uv, uo, 2 * VOV, 2 * OV, 2 * V), ix1(2));
                for (int sj = 0; sj < 2; ++sj)
                    for (int sk = 0; sk < 2; ++sk) {
                        const int sc = sj + sk - se;
                        if (sc < 0 || sc > 1) continue;
                        const double *B = t2s + se * VO2 + sc * O2 + sj * O + sk;
                        double *Cp = z3_.p + sa * V2O3 + sb * VO3 + si * O2 + sc * O3 + sj * O + sk;
                        gemm((int)(v * v * o), (int)(v * o * o), (int)v, -1.0, Av,
                             mv(B, ix3(uo, uo, 2 * O2, 2 * O, 2), ix1(2 * VO2)), 1.0,
                             ovw(Cp, ix3(uv, uo, 2 * V2O3, 2 * VO3, 2 * O2), ix3(uo, uo, 2 * O3, 2 * O, 2)),
                             -(560 + sa * 4 + sb * 2 + si), -(510 + se * 8 + sc * 4 + sj * 2 + sk), "T3_Q14");
                    }
            }
    for (int sa = 0; sa < 2; ++sa)
        for (int si = 0; si < 2; ++si)
            for (int sj = 0; sj < 2; ++sj) {
                const int sm = si + sj - sa;
                if (sm < 0 || sm > 1) continue;
                const MatView Av =
                    mv(x15_.p + sa * O3 + sm * O2 + si * O + sj, ix3(uo, uo, 2 * O3, 2 * O, 2), ix1(2 * O2));
                for (int sb = 0; sb < 2; ++sb)
                    for (int sc = 0; sc < 2; ++sc) {
                        const int sk = sb + sc - sm;
                        if (sk < 0 || sk > 1) continue;
                        const double *B = t2s + sb * VO2 + sc * O2 + sm * O + sk;
                        double *Cp = y3_.p + sa * V2O3 + si * O2 + sj * O + sb * VO3 + sc * O3 + sk;
                        gemm((int)(v * o * o), (int)(v * v * o), (int)o, 1.0, Av,
                             mv(B, ix3(uv, uo, 2 * VO2, 2 * O2, 2), ix1(2 * O)), 1.0,
                             ovw(Cp, ix3(uo, uo, 2 * V2O3, 2 * O2, 2 * O), ix3(uv, uo, 2 * VO3, 2 * O3, 2)),
                             -(570 + sa * 4 + si * 2 + sj), -(530 + sm * 8 + sb * 4 + sc * 2 + sk), "T3_Q15");
                    }
            }
}

// CCSDT-4 (ccsdt.cpp:1134-1180): terms of the previous t3 with X3 = 1/2 <ij||lm>,
// X4 = 1/2 <ab||de>, X6 = <al||id>, added to Y so that the assembly's P(a/bc) P(k/ij)
// produces them:
//   P(k/ij) sum_lm X3(i,j)(l,m) t3(abc,lmk): W is antisymmetric in abc, where P(a/bc) W = 3 W,
//     so Y += W / 3;
//   P(c/ab) sum_de X4(a,b)(d,e) t3(dec,ijk): W is antisymmetric in ab and ijk; with the cyclic
//     relabelling W'(a,b,c) = W(b,c,a), P(a/bc) W' = P(c/ab) W, and P(k/ij) W' = 3 W', so
//     Y(abc,ijk) += 1/3 sum_de X4(b,c)(d,e) t3(dea,ijk);
//   P(i/jk) P(a/bc) sum_ld X6(a,l)(i,d) t3(dbc,ljk): W is antisymmetric in bc and jk; with
//     W'(ijk) = W(kij), P(k/ij) W' = P(i/jk) W, so Y(abc,ijk) += sum_ld X6(a,l)(k,d) t3(dbc,lij).
void Engine::triples_m5_terms() {
    const int64_t o = o_, v = v_, O = 2 * o, V = 2 * v, O2 = O * O, O3 = O2 * O, VO3 = V * O3, V2O3 = V * VO3;
    const int64_t OV = O * V, O2V = O2 * V, V2 = V * V, VO2 = V * O2;
    const uint32_t uO = (uint32_t)O, uV = (uint32_t)V, uo = (uint32_t)o, uv = (uint32_t)v;
    const int iO = (int)O, iV = (int)V;
    const double *t3 = t3_.p;
    const double *X3 = so_oooo_.p, *X4 = so_vvvv_.p, *X6 = so_voov_.p;
    double a34 = 0.5 / 3.0;  // X3 = 1/2 <ij||lm>, X4 = 1/2 <ab||de>, times the 1/3 of the relabelling
    if (opt_.method >= CCSD_METHOD_CCSDT) {
        // CCSDT (ccsdt.cpp:1183-1200, 2128-2300), from this T1/T2 (tauso, t1so, and P2,
        // A1 + <lm||id> and E of triples_m4_terms):
        //   X3[i][j][l][m] = 1/2 <ij||lm> + 1/2 sum_d <lm||d e0> tau[d][e0][i][j]
        //                    - sum_d <lm||jd> t1[d][i] + sum_d <lm||id> t1[d][j]
        //     (e0 = the first virtual spin orbital: the reference's loop over (d,e) advances d)
        //   X4[a][b][d][e] = 1/2 <ab||de> + 1/2 sum_lm tau[a][b][l][m] <lm||de>
        //                    - sum_l <bl||de> t1[a][l] + sum_l <al||de> t1[b][l]
        //   X6[a][l][i][d] = <al||id> + P2[a][i][l][d] - sum_m t1[a][m] (A1 + <ml||id>)[m][l][i][d] + E[a][l][i][d]
        //   X7[i][m] = -1/2 sum_{l,d,e} <lm||de> tau[d][e][l][i] + sum_{l,d} <lm||id> t1[d][l]
        //   X8[a][e] = -sum_{l,d} <al||de> t1[d][l] - 1/2 sum_{l,m,d} <lm||de> tau[d][a][l][m] - sum_l f(l,e) t1[a][l]
        const MatView t1_xl = mv(t1so_.p, ix1(O), ix1(1)), t1_ie = mv(t1so_.p, ix1(1), ix1(O));
        axpby((int)O2, (int)O2, 0.5, mv(so_oooo_.p, ix1(O2), ix1(1)), 0.0, ovw(x3_.p, ix1(O2), ix1(1)));
        gemm((int)O2, (int)O2, iV, 0.5, mv(tauso_.p, ix1(1), ix1(VO2)), mv(so_oovv_.p, ix1(V2), ix1(V)), 1.0,
             ovw(x3_.p, ix1(O2), ix1(1)), 0, 0, "T3_X3_tau");
        gemm((int)O3, iO, iV, -1.0, mv(so_ooov_.p, ix1(V), ix1(1)), t1_ie, 1.0,
             ovw(x3_.p, ix3(uO, uO, O, 1, O2), ix1(O3)), 0, 0, "T3_X3_t1a");
        gemm((int)O3, iO, iV, 1.0, mv(so_ooov_.p, ix1(V), ix1(1)), t1_ie, 1.0,
             ovw(x3_.p, ix3(uO, uO, O, 1, O3), ix1(O2)), 0, 0, "T3_X3_t1b");
        axpby((int)V2, (int)V2, 0.5, mv(so_vvvv_.p, ix1(V2), ix1(1)), 0.0, ovw(x4_.p, ix1(V2), ix1(1)));
        gemm((int)V2, (int)V2, (int)O2, 0.5, mv(tauso_.p, ix1(O2), ix1(1)), mv(so_oovv_.p, ix1(1), ix1(V2)), 1.0,
             ovw(x4_.p, ix1(V2), ix1(1)), 0, 0, "T3_X4_tau");
        gemm((int)(V * V2), iV, iO, -1.0, mv(so_vovv_.p, ix2((uint32_t)V2, O * V2, 1), ix1(V2)), t1_xl, 1.0,
             ovw(x4_.p, ix1(1), ix1(V * V2)), 0, 0, "T3_X4_t1a");
        gemm((int)(V * V2), iV, iO, 1.0, mv(so_vovv_.p, ix2((uint32_t)V2, O * V2, 1), ix1(V2)), t1_xl, 1.0,
             ovw(x4_.p, ix2((uint32_t)V2, V * V2, 1), ix1(V2)), 0, 0, "T3_X4_t1b");
        copy(x6_.p, so_voov_.p, (size_t)(V * O2 * V));
        axpby((int)(V * O2), iV, 1.0, mv(p2_.p, ix3(uO, uO, O2V, V, OV), ix1(1)), 1.0,
              ovw(x6_.p, ix3(uO, uO, O2V, OV, V), ix1(1)));
        gemm((int)(O2 * V), iV, iO, -1.0, mv(a1_.p, ix1(1), ix1(O2V)), t1_xl, 1.0, ovw(x6_.p, ix1(1), ix1(O2V)), 0, 0,
             "T3_X6_t1C");
        axpby((int)(V * O2), iV, 1.0, mv(e15_.p, ix1(V), ix1(1)), 1.0, ovw(x6_.p, ix1(V), ix1(1)));
        gemm(iO, iO, (int)(O * V2), -0.5, mv(tauso_.p, ix1(1), ix2((uint32_t)V2, O, O2)),
             mv(so_oovv_.p, ix1(V2), ix2((uint32_t)V2, O * V2, 1)), 0.0, ovw(x7_.p, ix1(O), ix1(1)), 0, 0, "T3_X7_tau");
        gemm((int)O2, 1, (int)OV, 1.0, mv(so_ooov_.p, ix2(uO, V, OV), ix2(uV, O2V, 1)),
             mv(t1so_.p, ix1(0), ix2(uV, 1, O)), 1.0, ovw(x7_.p, ix1(1), ix1(0)), 0, 0, "T3_X7_t1");
        gemm((int)V2, 1, (int)OV, -1.0, mv(so_vovv_.p, ix2(uV, O * V2, 1), ix2(uV, V2, V)),
             mv(t1so_.p, ix1(0), ix2(uV, 1, O)), 0.0, ovw(x8_.p, ix1(1), ix1(0)), 0, 0, "T3_X8_t1");
        gemm(iV, iV, (int)VO2, -0.5, mv(tauso_.p, ix1(O2), ix2((uint32_t)O2, VO2, 1)),
             mv(so_oovv_.p, ix1(1), ix2((uint32_t)O2, V, V2)), 1.0, ovw(x8_.p, ix1(V), ix1(1)), 0, 0, "T3_X8_tau");
        k_t1_spin((int)o, (int)v, f_ov_.p, fsoT_.p, st_);  // fsoT[e][l] = f(l,e) in spin orbitals
        gemm(iV, iV, iO, -1.0, t1_xl, mv(fsoT_.p, ix1(O), ix1(1)), 1.0, ovw(x8_.p, ix1(V), ix1(1)), 0, 0, "T3_X8_f");
        // P(a/bc) sum_d X8(a,d) t3(dbc,ijk): antisymmetric in ijk, so Y += 1/3 of it. X8 is
        // spin-diagonal, but one contraction per spin leaves nvir rows, under half of a 64-row
        // FP64 tile, so the dense form is faster
        gemm(iV, (int)(V2 * O3), iV, 1.0 / 3.0, mv(x8_.p, ix1(V), ix1(1)), mv(t3, ix1(1), ix1(V2O3)), 1.0,
             ovw(y3_.p, ix1(V2O3), ix1(1)), 0, 0, "T3_X8t3");
        // P(i/jk) sum_m X7(i,m) t3(abc,mjk): as the X6 term, Y(abc,ijk) += 1/3 sum_m X7(k,m) t3(abc,mij)
        gemm((int)(V * V2 * O2), iO, iO, 1.0 / 3.0, mv(t3, ix2((uint32_t)O2, O3, 1), ix1(O2)), mv(x7_.p, ix1(O), ix1(1)),
             1.0, ovw(y3_.p, ix2((uint32_t)O2, O3, O), ix1(1)), 0, 0, "T3_X7t3");
        X3 = x3_.p;
        X4 = x4_.p;
        X6 = x6_.p;
        a34 = 1.0 / 3.0;  // the dressed X3, X4 carry their 1/2
    }
    // The X4, X3 and X6 terms by spin blocks. Each intermediate conserves spin, so of the
    // 16 spin assignments of its four indices 6 are non-zero. A pair of spin-orbital
    // indices with strides P, Q at total spin 0 or 2 is one spin pair; at total spin 1 the
    // two pairs (0,1), (1,0) sit at Q and P, one index q at Q + q (P - Q), so they merge
    // into one contraction. The indices of t3 outside the blocks stay dense (t3 is zero
    // where their spins do not balance).
    struct Pair {
        uint32_t n;
        int64_t base, step;
    };
    auto pair = [](int s, int64_t P, int64_t Q) {
        return s == 0 ? Pair{1, 0, 0} : s == 1 ? Pair{2, Q, P - Q} : Pair{1, P + Q, 0};
    };
    // X4: Y[a][b][c][ijk] += a34 sum_{d,e} X4[b][c][d][e] t3[d][e][a][ijk]: M = (q, b', c'),
    // N = (a', ijk) at each spin of a, K = (q, d', e'), sb + sc = sd + se
    for (int sp = 0; sp < 3; ++sp) {
        const Pair bcX = pair(sp, V * V2, V2), deX = pair(sp, V, 1), deT = pair(sp, V2O3, VO3), bcY = pair(sp, VO3, O3);
        for (int sa = 0; sa < 2; ++sa)
            gemm((int)(bcX.n * v * v), (int)(v * O3), (int)(deX.n * v * v), a34,
                 mv(X4 + bcX.base + deX.base, ix3(uv, uv, bcX.step, 2 * V * V2, 2 * V2),
                    ix3(uv, uv, deX.step, 2 * V, 2)),
                 mv(t3 + sa * O3 + deT.base, ix2((uint32_t)O3, 2 * O3, 1), ix3(uv, uv, deT.step, 2 * V2O3, 2 * VO3)),
                 1.0,
                 ovw(y3_.p + bcY.base + sa * V2O3, ix3(uv, uv, bcY.step, 2 * VO3, 2 * O3),
                     ix2((uint32_t)O3, 2 * V2O3, 1)),
                 0, 0, "T3_X4t3");
    }
    // X3: Y[abc][i][j][k] += a34 sum_{l,m} X3[i][j][l][m] t3[abc][l][m][k]: M = (abc, k),
    // N = (q, i', j'), K = (q, l', m'), si + sj = sl + sm
    for (int sp = 0; sp < 3; ++sp) {
        const Pair ijX = pair(sp, O * O2, O2), lmX = pair(sp, O, 1), lmT = pair(sp, O2, O), ijY = pair(sp, O2, O);
        gemm((int)(V * V2 * O), (int)(ijX.n * o * o), (int)(lmX.n * o * o), a34,
             mv(t3 + lmT.base, ix2(uO, O3, 1), ix3(uo, uo, lmT.step, 2 * O2, 2 * O)),
             mv(X3 + ijX.base + lmX.base, ix3(uo, uo, ijX.step, 2 * O * O2, 2 * O2), ix3(uo, uo, lmX.step, 2 * O, 2)),
             1.0, ovw(y3_.p + ijY.base, ix2(uO, O3, 1), ix3(uo, uo, ijY.step, 2 * O2, 2 * O)), 0, 0, "T3_X3t3");
    }
    // X6: Y[a][bc][ij][k] += sum_{l,d} X6[a][l][k][d] t3[d][bc][l][ij]: M = (a,k), N = (bc, ij),
    // K = (l,d), sa + sl = sk + sd. sa = sk (then sl = sd) is one contraction over q = sa,
    // q' = sl; sa != sk fixes all four spins (sd = sa, sl = sk).
    gemm((int)(2 * v * o), (int)(V2 * O2), (int)(2 * o * v), 1.0,
         mv(X6, ix3(uv, uo, O2V + V, 2 * O2V, 2 * V), ix3(uo, uv, OV + 1, 2 * OV, 2)),
         mv(t3, ix2((uint32_t)O2, O3, 1), ix3(uo, uv, O2 + V2O3, 2 * O2, 2 * V2O3)), 1.0,
         ovw(y3_.p, ix3(uv, uo, V2O3 + 1, 2 * V2O3, 2), ix2((uint32_t)O2, O3, O)), 0, 0, "T3_X6t3");
    for (int sa = 0; sa < 2; ++sa) {
        const int sk = 1 - sa, sl = 1 - sa, sd = sa;
        gemm((int)(v * o), (int)(V2 * O2), (int)(o * v), 1.0,
             mv(X6 + sa * O2V + sk * V + sl * OV + sd, ix2(uo, 2 * O2V, 2 * V), ix2(uv, 2 * OV, 2)),
             mv(t3 + sl * O2 + sd * V2O3, ix2((uint32_t)O2, O3, 1), ix2(uv, 2 * O2, 2 * V2O3)), 1.0,
             ovw(y3_.p + sa * V2O3 + sk, ix2(uo, 2 * V2O3, 2), ix2((uint32_t)O2, O3, O)), 0, 0, "T3_X6t3");
    }
}

void Engine::triples_step() {
    const int64_t o = o_, v = v_, O = 2 * o, V = 2 * v, O2 = O * O, O3 = O2 * O, VO3 = V * O3, V2O3 = V * VO3;
    const int io = (int)o, iv = (int)v;
    const double *t3 = t3_.p;
    k_t2_spin(io, iv, t2_.p, t2so_.p, st_);

    // ---- the previous T3 into the alpha-beta numerators (ccsdt.cpp:419-434, 640-670)
    // R1[i][a] += 1/4 sum_{b,c,jk} <jk||bc> t3[2a][b][c][2i][j][k]
    gemm(io * iv, 1, (int)(V * V * O2), 0.25,
         mv(t3, ix2((uint32_t)v, 2 * O2, 2 * V2O3), ix3((uint32_t)V, (uint32_t)O2, VO3, O3, 1)),
         mv(so_oovv_.p, ix1(0), ix3((uint32_t)V, (uint32_t)O2, V, 1, V * V)), 1.0,
         ovw(R1_.p, ix2((uint32_t)v, v, 1), ix1(0)), 0, 0, "R1_T3");
    // R[i][j][a][b] (a = 2a', b = 2b'+1, i = 2i', j = 2j'+1) from the previous t3, by
    // spin blocks of the summed indices (3 of the 8 spin triples conserve spin):
    struct Spins {
        int s0, s1, s2;
    };
    const uint32_t uo = (uint32_t)o, uv = (uint32_t)v;
    const Dim rows_ija = ix3(uo, uv, 2 * O2, 2 * O, 2 * V2O3);  // t3 rows (i', j', a') at fixed spins
    const Dim rows_iab = ix3(uv, uv, 2 * O2, 2 * V2O3, 2 * VO3);
    //   + 1/2 sum_{c,d,k} <bk||cd> t3[a][c][d][i][j][k]    (sc + sd = 1 + sk)
    const Spins vb[3] = {{0, 1, 0}, {1, 0, 0}, {1, 1, 1}};
    //   - 1/2 sum_{c,d,k} <ak||cd> t3[b][c][d][i][j][k]    (sc + sd = sk)
    const Spins va[3] = {{0, 0, 0}, {0, 1, 1}, {1, 0, 1}};
    for (int q = 0; q < 3; ++q) {
        const Dim K_cdk = ix3(uv, uo, 2 * VO3, 2 * O3, 2);   // (c', d', k') in t3
        const Dim Kv_cdk = ix3(uv, uo, 2 * V, 2, 2 * V * V);  // (c', d', k') in <bk||cd>
        const OutView Rb = ovw(R_.p, ix3(uo, uv, o * v * v, v * v, v), ix1(1));
        const OutView Ra = ovw(R_.p, ix3(uo, uv, o * v * v, v * v, 1), ix1(v));
        {
            const Spins &sp = vb[q];
            const int64_t t3o = sp.s0 * VO3 + sp.s1 * O3 + sp.s2, io_ = sp.s0 * V + sp.s1 + sp.s2 * V * V;
            gemm(io * io * iv, iv, (int)(v * v * o), 0.5, mv(t3 + O + t3o, rows_ija, K_cdk),
                 mv(so_vovv_.p + O * V * V + io_, ix1(2 * O * V * V), Kv_cdk), 1.0, Rb, 0, 400 + q, "R2_T3_vovv_b");
        }
        {
            const Spins &sp = va[q];
            const int64_t t3o = sp.s0 * VO3 + sp.s1 * O3 + sp.s2, io_ = sp.s0 * V + sp.s1 + sp.s2 * V * V;
            gemm(io * io * iv, iv, (int)(v * v * o), -0.5, mv(t3 + V2O3 + O + t3o, rows_ija, K_cdk),
                 mv(so_vovv_.p + io_, ix1(2 * O * V * V), Kv_cdk), 1.0, Ra, 0, 403 + q, "R2_T3_vovv_a");
        }
    }
    //   - 1/2 sum_{c,k,m} <km||jc> t3[a][b][c][i][k][m]    (sk + sm = 1 + sc)
    const Spins oj[3] = {{0, 0, 1}, {0, 1, 0}, {1, 1, 1}};
    //   + 1/2 sum_{c,k,m} <km||ic> t3[a][b][c][j][k][m]    (sk + sm = sc)
    const Spins oi[3] = {{0, 0, 0}, {1, 0, 1}, {1, 1, 0}};
    for (int q = 0; q < 3; ++q) {
        const Dim K_ckm = ix3(uo, uo, 2 * O3, 2 * O, 2);              // (c', k', m') in t3
        const Dim Ko_ckm = ix3(uo, uo, 2, 2 * O2 * V, 2 * O * V);     // (c', k', m') in <km||jc>
        {
            const Spins &sp = oj[q];
            const int64_t t3o = sp.s0 * O3 + sp.s1 * O + sp.s2, io_ = sp.s0 + sp.s1 * O2 * V + sp.s2 * O * V;
            gemm(io * iv * iv, io, (int)(v * o * o), -0.5, mv(t3 + VO3 + t3o, rows_iab, K_ckm),
                 mv(so_ooov_.p + V + io_, ix1(2 * V), Ko_ckm), 1.0,
                 ovw(R_.p, ix3(uv, uv, o * v * v, v, 1), ix1(v * v)), 0, 406 + q, "R2_T3_ooov_j");
        }
        {
            const Spins &sp = oi[q];
            const int64_t t3o = sp.s0 * O3 + sp.s1 * O + sp.s2, io_ = sp.s0 + sp.s1 * O2 * V + sp.s2 * O * V;
            gemm(io * iv * iv, io, (int)(v * o * o), 0.5, mv(t3 + VO3 + O2 + t3o, rows_iab, K_ckm),
                 mv(so_ooov_.p + io_, ix1(2 * V), Ko_ckm), 1.0,
                 ovw(R_.p, ix3(uv, uv, v * v, v, 1), ix1(o * v * v)), 0, 409 + q, "R2_T3_ooov_i");
        }
    }

    if (opt_.method >= CCSD_METHOD_CCSDT1B) triples_1b_terms();  // also from the previous t3
    // Full CCSDT: the reference's X3 tau loop (ccsdt.cpp:2199-2206) advances d with e fixed
    // at the first virtual, so its T3, and with it the T3 terms above, break the alpha/beta
    // symmetry; the closed-shell t2 keeps one amplitude per pair t2[ij][ab] = t2[ji][ba],
    // here the mean of the two alpha-beta numerators
    if (opt_.method >= CCSD_METHOD_CCSDT) k_pair_mean(io, iv, R_.p, st_);

    // CCSDT-2 dresses X1 and X2 with this T2 (ccsdt.cpp:1960-2040):
    //   X1[b][c][e][k] = <bc||ek> + 1/2 sum_lm <lm||ek> t2so[b][c][l][m],  <lm||ek> = -<lm||ke>
    //   X2[m][c][j][k] = <mc||jk> + 1/2 sum_de t2so[d][e][j][k] <mc||de>,  <mc||de> = -<cm||de>
    const bool m3 = opt_.method >= CCSD_METHOD_CCSDT2;
    const double *X1 = so_vvvo_.p, *X2 = so_ovoo_.p;
    if (m3) {
        copy(x1d_.p, so_vvvo_.p, (size_t)(V * V * V * O));
        gemm((int)(V * V), (int)(V * O), (int)O2, -0.5, mv(t2so_.p, ix1(O2), ix1(1)),
             mv(so_ooov_.p, ix2((uint32_t)O, 1, V), ix1(O * V)), 1.0, ovw(x1d_.p, ix1(V * O), ix1(1)), 0, 0,
             "T3_X1_dress");
        copy(x2d_.p, so_ovoo_.p, (size_t)(O * V * O2));
        gemm((int)(O * V), (int)O2, (int)(V * V), -0.5, mv(so_vovv_.p, ix2((uint32_t)V, V * V, O * V * V), ix1(1)),
             mv(t2so_.p, ix1(1), ix1(O2)), 1.0, ovw(x2d_.p, ix1(O2), ix1(1)), 0, 0, "T3_X2_dress");
        X1 = x1d_.p;
        X2 = x2d_.p;
    }
    if (opt_.method >= CCSD_METHOD_CCSDT) {  // T3 terms of X1 and X2 (ccsdt.cpp:1982-1988, 2020-2030)
        const uint32_t uO = (uint32_t)O, uV = (uint32_t)V, uo = (uint32_t)o, uv = (uint32_t)v;
        const int64_t OV2 = O * V * V, V2 = V * V;
        // By the 6 spin blocks of <lm||de> (sl + sm = sd + se); the other indices of t3 stay dense.
        for (int sd = 0; sd < 2; ++sd)
            for (int se = 0; se < 2; ++se)
                for (int sl = 0; sl < 2; ++sl) {
                    const int sm = sd + se - sl;
                    if (sm < 0 || sm > 1) continue;
                    const double *g = so_oovv_.p + sl * OV2 + sm * V2 + sd * V + se;  // <lm||de> at [l][m][d][e]
                    // X1[b][c][d][k] -= 1/2 sum_{l,m,e} <lm||de> t3[b][e][c][l][m][k]:
                    // M = (b,c,k), N = d', K = (e', l', m')
                    gemm((int)(V * V * O), iv, (int)(v * o * o), -0.5,
                         mv(t3 + se * VO3 + sl * O2 + sm * O, ix3(uV, uO, V2O3, O3, 1), ix3(uo, uo, 2 * VO3, 2 * O2, 2 * O)),
                         mv(g, ix1(2 * V), ix3(uo, uo, 2, 2 * OV2, 2 * V2)), 1.0,
                         ovw(x1d_.p + sd * O, ix3(uV, uO, V * V * O, V * O, 1), ix1(2 * O)), 0, 0, "T3_X1_t3");
                    // X2[l][c][j][k] += 1/2 sum_{m,d,e} <lm||de> t3[d][e][c][j][m][k]:
                    // M = (c,j,k), N = l', K = (d', e', m')
                    gemm((int)(V * O2), io, (int)(v * v * o), 0.5,
                         mv(t3 + sd * V2O3 + se * VO3 + sm * O, ix3(uO, uO, O3, O2, 1),
                            ix3(uv, uo, 2 * V2O3, 2 * VO3, 2 * O)),
                         mv(g, ix1(2 * OV2), ix3(uv, uo, 2 * V, 2, 2 * V2)), 1.0,
                         ovw(x2d_.p + sl * V * O2, ix1(1), ix1(2 * V * O2)), 0, 0, "T3_X2_t3");
                }
    }
    // integral operands are split once (positive keys) unless they change every update
    const int ksign = m3 ? -1 : 1;
    // The Y blocks below write only their 18 spin blocks and leave the rest of Y at zero;
    // the CCSDT-4 terms add to all of Y (also to spin-allowed elements outside those
    // blocks), so Y starts from zero each update there
    if (opt_.method >= CCSD_METHOD_CCSDT4) y3_.zero(st_);

    // ---- T3 from the previous T2 (ccsdt.cpp:1016-1058, 1235-1238), by spin blocks.
    // Spin orbital X = 2x + s, so a block of fixed spins is a stride-2 view of
    // spatial indices.  t2so and the integral blocks conserve spin, so of the
    // 2^7 spin assignments of each product only 18 are non-zero; each is one
    // contraction over spatial indices (1/7 of the dense spin-orbital flops).  The
    // other blocks of Y and Z are zero and stay at the zero set in triples_setup.
    for (int sa = 0; sa < 2; ++sa)
        for (int si = 0; si < 2; ++si)
            for (int sj = 0; sj < 2; ++sj) {
                // Y[a][b][c][i][j][k] = sum_e t2so[a][e][i][j] <bc||ek>: se = si + sj - sa,
                // (sb, sc, sk) with sb + sc = se + sk;  M = (a,i,j), N = (b,c,k), K = e (spatial)
                const int se = si + sj - sa;
                if (se < 0 || se > 1) continue;
                const double *A = t2so_.p + sa * V * O2 + se * O2 + si * O + sj;
                const MatView Av = mv(A, ix3(uo, uo, 2 * V * O2, 2 * O, 2), ix1(2 * O2));
                for (int sb = 0; sb < 2; ++sb)
                    for (int sc = 0; sc < 2; ++sc) {
                        const int sk = sb + sc - se;
                        if (sk < 0 || sk > 1) continue;
                        const double *B = X1 + sb * V * V * O + sc * V * O + se * O + sk;
                        double *Cp = y3_.p + sa * V2O3 + si * O2 + sj * O + sb * VO3 + sc * O3 + sk;
                        gemm((int)(v * o * o), (int)(v * v * o), (int)v, 1.0, Av,
                             mv(B, ix3(uv, uo, 2 * V * V * O, 2 * V * O, 2), ix1(2 * O)), 0.0,
                             ovw(Cp, ix3(uo, uo, 2 * V2O3, 2 * O2, 2 * O), ix3(uv, uo, 2 * VO3, 2 * O3, 2)),
                             -(300 + sa * 4 + si * 2 + sj), ksign * (310 + se * 8 + sb * 4 + sc * 2 + sk), "T3_Y");
                    }
            }
    for (int sa = 0; sa < 2; ++sa)
        for (int sb = 0; sb < 2; ++sb)
            for (int si = 0; si < 2; ++si) {
                // Z[a][b][c][i][j][k] = sum_m t2so[a][b][i][m] <mc||jk>: sm = sa + sb - si,
                // (sc, sj, sk) with sm + sc = sj + sk;  M = (a,b,i), N = (c,j,k), K = m (spatial)
                const int sm = sa + sb - si;
                if (sm < 0 || sm > 1) continue;
                const double *A = t2so_.p + sa * V * O2 + sb * O2 + si * O + sm;
                const MatView Av = mv(A, ix3(uv, uo, 2 * V * O2, 2 * O2, 2 * O), ix1(2));
                for (int sj = 0; sj < 2; ++sj)
                    for (int sk = 0; sk < 2; ++sk) {
                        const int sc = sj + sk - sm;
                        if (sc < 0 || sc > 1) continue;
                        const double *B = X2 + sm * V * O2 + sc * O2 + sj * O + sk;
                        double *Cp = z3_.p + sa * V2O3 + sb * VO3 + si * O2 + sc * O3 + sj * O + sk;
                        gemm((int)(v * v * o), (int)(v * o * o), (int)o, 1.0, Av,
                             mv(B, ix3(uo, uo, 2 * O2, 2 * O, 2), ix1(2 * V * O2)), 0.0,
                             ovw(Cp, ix3(uv, uo, 2 * V2O3, 2 * VO3, 2 * O2), ix3(uo, uo, 2 * O3, 2 * O, 2)),
                             -(330 + sa * 4 + sb * 2 + si), ksign * (340 + sm * 8 + sc * 4 + sj * 2 + sk), "T3_Z");
                    }
            }
    if (m3) triples_m3_products();
    if (opt_.method >= CCSD_METHOD_CCSDT4) triples_m5_terms();  // the previous t3 into Y

    cudaEvent_t ea = nullptr, eb = nullptr, ec = nullptr;
    if (opt_.profile) {  // a site of its own in the contraction profile (no flops)
        ea = prof_event();
        eb = prof_event();
        ec = prof_event();
        CCSD_CUDA(cudaEventRecord(ea, st_));
        CCSD_CUDA(cudaEventRecord(eb, st_));
    }
    k_t3_assemble(io, iv, y3_.p, z3_.p, m3 ? q12_.p : nullptr, m3 ? q13_.p : nullptr, eo_.p, ev_.p, t3_.p, st_);
    if (opt_.profile) {
        CCSD_CUDA(cudaEventRecord(ec, st_));
        prof_pending_.push_back(ProfPending{"T3_assemble", ea, eb, ec, 0.0, false});
    }
}

}  // namespace ccsd
