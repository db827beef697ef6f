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
    for (int kind = 0; kind < 5; ++kind) k_so_block(kind, o_, v_, ovov_.p, ovoo_.p, ovvv_.p, blocks[kind]->p, st_);
    t3_.zero(st_);  // T3 starts at zero (the first update is CCSD-like)
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
    // R[i][j][a][b] += 1/2 sum_{c,d,k} <bk||cd> t3[a][c][d][i][j][k]   (a = 2a', b = 2b'+1, i = 2i', j = 2j'+1)
    const Dim K_cdk = ix3((uint32_t)V, (uint32_t)O, VO3, O3, 1);
    const Dim Kv_cdk = ix3((uint32_t)V, (uint32_t)O, V, 1, V * V);
    gemm(io * io * iv, iv, (int)(V * V * O), 0.5, mv(t3 + O, ix3((uint32_t)o, (uint32_t)v, 2 * O2, 2 * O, 2 * V2O3), K_cdk),
         mv(so_vovv_.p + O * V * V, ix1(2 * O * V * V), Kv_cdk), 1.0,
         ovw(R_.p, ix3((uint32_t)o, (uint32_t)v, o * v * v, v * v, v), ix1(1)), 0, 23, "R2_T3_vovv_b");
    // - 1/2 sum_{c,d,k} <ak||cd> t3[b][c][d][i][j][k]
    gemm(io * io * iv, iv, (int)(V * V * O), -0.5,
         mv(t3 + V2O3 + O, ix3((uint32_t)o, (uint32_t)v, 2 * O2, 2 * O, 2 * V2O3), K_cdk),
         mv(so_vovv_.p, ix1(2 * O * V * V), Kv_cdk), 1.0,
         ovw(R_.p, ix3((uint32_t)o, (uint32_t)v, o * v * v, v * v, 1), ix1(v)), 0, 24, "R2_T3_vovv_a");
    // - 1/2 sum_{c,km} <km||jc> t3[a][b][c][i][k][m]
    const Dim K_ckm = ix2((uint32_t)O2, O3, 1);
    const Dim Ko_ckm = ix2((uint32_t)O2, 1, O * V);
    gemm(io * iv * iv, io, (int)(V * O2), -0.5,
         mv(t3 + VO3, ix3((uint32_t)v, (uint32_t)v, 2 * O2, 2 * V2O3, 2 * VO3), K_ckm),
         mv(so_ooov_.p + V, ix1(2 * V), Ko_ckm), 1.0,
         ovw(R_.p, ix3((uint32_t)v, (uint32_t)v, o * v * v, v, 1), ix1(v * v)), 0, 25, "R2_T3_ooov_j");
    // + 1/2 sum_{c,km} <km||ic> t3[a][b][c][j][k][m]
    gemm(io * iv * iv, io, (int)(V * O2), 0.5,
         mv(t3 + VO3 + O2, ix3((uint32_t)v, (uint32_t)v, 2 * O2, 2 * V2O3, 2 * VO3), K_ckm),
         mv(so_ooov_.p, ix1(2 * V), Ko_ckm), 1.0,
         ovw(R_.p, ix3((uint32_t)v, (uint32_t)v, v * v, v, 1), ix1(o * v * v)), 0, 26, "R2_T3_ooov_i");

    // ---- T3 from the previous T2 (ccsdt.cpp:1016-1058, 1235-1238)
    // Y[a][b][c][i][j][k] = sum_e t2so[a][e][i][j] <bc||ek>:  M = (a,i,j), N = (b,c,k), K = e
    gemm((int)(V * O2), (int)(V * V * O), (int)V, 1.0,
         mv(t2so_.p, ix3((uint32_t)O, (uint32_t)O, V * O2, O, 1), ix1(O2)),
         mv(so_vvvo_.p, ix3((uint32_t)V, (uint32_t)O, V * V * O, V * O, 1), ix1(O)), 0.0,
         ovw(y3_.p, ix3((uint32_t)O, (uint32_t)O, V2O3, O2, O), ix3((uint32_t)V, (uint32_t)O, VO3, O3, 1)), -21, 21,
         "T3_Y");
    // Z[a][b][c][i][j][k] = sum_m t2so[a][b][i][m] <mc||jk>:  M = (a,b,i), N = (c,j,k), K = m
    gemm((int)(V * V * O), (int)(V * O2), (int)O, 1.0,
         mv(t2so_.p, ix3((uint32_t)V, (uint32_t)O, V * O2, O2, O), ix1(1)),
         mv(so_ovoo_.p, ix3((uint32_t)O, (uint32_t)O, O2, O, 1), ix1(V * O2)), 0.0,
         ovw(z3_.p, ix3((uint32_t)V, (uint32_t)O, V2O3, VO3, O2), ix3((uint32_t)O, (uint32_t)O, O3, O, 1)), -22, 22,
         "T3_Z");
    k_t3_assemble(io, iv, y3_.p, z3_.p, eo_.p, ev_.p, t3_.p, st_);
}

}  // namespace ccsd
