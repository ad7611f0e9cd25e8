// GENERATED by finite_root_generation_gb300/gen/gen_system.py -- do not edit.
//
// One j-group of the Stephenson II loop-closure system (reference FSYS,
// htpykinematics.cu:36-122): the three equations (rows j-1, j+6, j+13), their
// nonzero partial derivatives over Z (JVAR's sparsity, htpykinematics.cu:129-1129)
// and the t-derivative dF/dq . dq/dt (JH's last column, htpysupport.cu:113-121).
// Straight-line cost per group: 352 complex mul, 239 complex add/sub,
// 5 real-scalar x complex.
#pragma once

#define FRG_GEN_CMUL 352
#define FRG_GEN_CADD 239
#define FRG_GEN_SMUL 5

// Output slots: fI, dI[8] over {A,C,H,Ac,Cc,Hc,U_j,Z0}, tI;
//               fII, dII[6] over {B,F,Bc,Fc,U_j,Z0}, tII;
//               fIII, dIII[16] over {A..H,Ac..Hc,U_j,Z0}, tIII.
template <typename T>
struct FrgGroupOut {
  cx<T> fI, dI[8], tI;
  cx<T> fII, dII[6], tII;
  cx<T> fIII, dIII[16], tIII;
};

// Column in Z of each derivative slot (U_j's column is 13 + j, marked -1).
#define FRG_COLS_I {0, 2, 6, 7, 9, 13, -1, 21}
#define FRG_COLS_II {1, 4, 8, 11, -1, 21}
#define FRG_COLS_III {0, 1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12, 13, -1, 21}

template <typename T>
__device__ __forceinline__ void frg_group_eval(
    const cx<T> A, const cx<T> B, const cx<T> C, const cx<T> D, const cx<T> F, const cx<T> G,
    const cx<T> H, const cx<T> Ac, const cx<T> Bc, const cx<T> Cc, const cx<T> Dc, const cx<T> Fc,
    const cx<T> Gc, const cx<T> Hc, const cx<T> z,
    const cx<T> e1, const cx<T> e2, const cx<T> ec1, const cx<T> ec2,
    const cx<T> z2, const cx<T> z3,
    const cx<T> P0, const cx<T> Pc0, const cx<T> dP0, const cx<T> dPc0,
    const cx<T> U, const cx<T> iU, const cx<T> Pj, const cx<T> Pcj, const cx<T> Qj, const cx<T> Qcj,
    const cx<T> dPj, const cx<T> dPcj, const cx<T> dQj, const cx<T> dQcj,
    FrgGroupOut<T>& o) {
  const cx<T> x0 = P0*Pc0 + Pcj*Pj;
  const cx<T> x1 = x0*z3;
  const cx<T> x2 = Pc0*z;
  const cx<T> x3 = (-(x2));
  const cx<T> x4 = Cc + x3;
  const cx<T> x5 = x4*z;
  const cx<T> x6 = P0*z;
  const cx<T> x7 = (-(x6));
  const cx<T> x8 = C + x7;
  const cx<T> x9 = Hc*z;
  const cx<T> x10 = (-(Ac));
  const cx<T> x11 = Pcj*z;
  const cx<T> x12 = x10 + x11;
  const cx<T> x13 = Cc + x12;
  const cx<T> x14 = x13*z;
  const cx<T> x15 = (-(A));
  const cx<T> x16 = Pj*z;
  const cx<T> x17 = x15 + x16;
  const cx<T> x18 = C + x17;
  const cx<T> x19 = Ac*z;
  const cx<T> x20 = Ac - Cc;
  const cx<T> x21 = Qcj*x20;
  const cx<T> x22 = (-(x16));
  const cx<T> x23 = A + x22;
  const cx<T> x24 = x23*z;
  const cx<T> x25 = A - C;
  const cx<T> x26 = Qj*x25;
  const cx<T> x27 = (-(x11));
  const cx<T> x28 = Ac + x27;
  const cx<T> x29 = x28*z;
  const cx<T> x30 = (-x12) - x21;
  const cx<T> x31 = H + x7;
  const cx<T> x32 = U*x31;
  const cx<T> x33 = (-x17) - x26;
  const cx<T> x34 = Hc + x3;
  const cx<T> x35 = iU*x34;
  const cx<T> x36 = x35*z2;
  const cx<T> x37 = Qj*x29;
  const cx<T> x38 = (-cx<T>(T(1.0))) + Qj;
  const cx<T> x39 = x28 - Qcj*x20;
  const cx<T> x40 = U*x39;
  const cx<T> x41 = A*z;
  const cx<T> x42 = Qcj*x24;
  const cx<T> x43 = (-cx<T>(T(1.0))) + Qcj;
  const cx<T> x44 = (-(Qj*x25));
  const cx<T> x45 = x23 + x44;
  const cx<T> x46 = iU*x45;
  const cx<T> x47 = x46*z2;
  const cx<T> x48 = z2*(iU*iU);
  const cx<T> x49 = (T(3.0)*(x0*z2));
  const cx<T> x50 = Pj*z2;
  const cx<T> x51 = iU*z2;
  const cx<T> x52 = Pc0*z3;
  const cx<T> x53 = P0*z3;
  const cx<T> x54 = Pj*z3;
  const cx<T> x55 = Pcj*z3;
  const cx<T> x56 = Bc + x3;
  const cx<T> x57 = x56*z;
  const cx<T> x58 = B + x7;
  const cx<T> x59 = Fc*z;
  const cx<T> x60 = B*Pcj + Bc*Pj;
  const cx<T> x61 = Bc + x27;
  const cx<T> x62 = F + x7;
  const cx<T> x63 = B + x22;
  const cx<T> x64 = Fc + x3;
  const cx<T> x65 = x51*x64;
  const cx<T> x66 = U*x61;
  const cx<T> x67 = U*x62;
  const cx<T> x68 = x51*x63;
  const cx<T> x69 = iU*z3;
  const cx<T> x70 = (-(G));
  const cx<T> x71 = D + x70;
  const cx<T> x72 = (-(Gc));
  const cx<T> x73 = Dc + x72;
  const cx<T> x74 = x73*z;
  const cx<T> x75 = B - D;
  const cx<T> x76 = e1*x75;
  const cx<T> x77 = C + x70;
  const cx<T> x78 = e2*x77;
  const cx<T> x79 = x62*x76 - x31*x78;
  const cx<T> x80 = Bc - Dc;
  const cx<T> x81 = ec1*x80;
  const cx<T> x82 = Cc + x72;
  const cx<T> x83 = ec2*x82;
  const cx<T> x84 = x64*x81 - x34*x83;
  const cx<T> x85 = x79*x84;
  const cx<T> x86 = ec2*x39;
  const cx<T> x87 = Bc + x10 + x21 + x61*x81 - x82*x86;
  const cx<T> x88 = U*x79;
  const cx<T> x89 = e2*x45;
  const cx<T> x90 = B + x15 + x26 + x63*x76 - x77*x89;
  const cx<T> x91 = x51*x84;
  const cx<T> x92 = x87*z;
  const cx<T> x93 = x91 - x92;
  const cx<T> x94 = x84*z;
  const cx<T> x95 = e1*x63;
  const cx<T> x96 = cx<T>(T(1.0)) + x76 + x95;
  const cx<T> x97 = (-(x84));
  const cx<T> x98 = x97*z;
  const cx<T> x99 = x62*x98;
  const cx<T> x100 = (-(x87));
  const cx<T> x101 = x100*x67;
  const cx<T> x102 = x100*z;
  const cx<T> x103 = x101 - x99 + x68*x97 - x102*x63;
  const cx<T> x104 = x32*x87;
  const cx<T> x105 = Qj + x89 + Qj*x78;
  const cx<T> x106 = x51*x97;
  const cx<T> x107 = U*x100;
  const cx<T> x108 = x100*x32;
  const cx<T> x109 = x90*z;
  const cx<T> x110 = x88 - x109;
  const cx<T> x111 = (-(e2*x77));
  const cx<T> x112 = (-x111*x31) - x62*x76;
  const cx<T> x113 = (-(x80));
  const cx<T> x114 = (-(x113*x61));
  const cx<T> x115 = (-(x64*x80));
  const cx<T> x116 = (-(e1*x75));
  const cx<T> x117 = A + x44 - B + x116*x63 - x111*x45;
  const cx<T> x118 = U*x112*x114 + x112*x115*z - x114*x117*z - x115*x117*x51;
  const cx<T> x119 = ec1*x61;
  const cx<T> x120 = cx<T>(T(1.0)) + x119 + x81;
  const cx<T> x121 = (-(x79));
  const cx<T> x122 = U*x121;
  const cx<T> x123 = (-(x90));
  const cx<T> x124 = x121*z;
  const cx<T> x125 = ec1*x123*x65 - ec1*x124*x64;
  const cx<T> x126 = Qcj + x86 + Qcj*x83;
  const cx<T> x127 = x36*x90;
  const cx<T> x128 = x71*z;
  const cx<T> x129 = x123*z;
  const cx<T> x130 = x121*x40;
  const cx<T> x131 = x123*x36;
  const cx<T> x132 = x76 - x78;
  const cx<T> x133 = x81 - x83;
  const cx<T> x134 = (-(x133));
  const cx<T> x135 = (-(x132));
  const cx<T> x136 = U*x87;
  const cx<T> x137 = x51*x90;
  o.fI = (-x1) + A*x14 + x18*x19 + x21*x24 + x26*x29 + x30*x32 + x33*x36 - H*x5 - x8*x9;
  o.dI[0] = x14 + x37 - x19 + x21*z - x36*x38;
  o.dI[1] = x19 - x37 - x9 + Qj*x36;
  o.dI[2] = x40 - x5;
  o.dI[3] = x42 - x41 + x18*z + x26*z - x32*x43;
  o.dI[4] = x41 - x42 + Qcj*x32 - H*z;
  o.dI[5] = x47 - x8*z;
  o.dI[6] = x31*x39 - x34*x45*x48;
  o.dI[7] = (-x49) + A*x11 + A*x13 + Ac*x16 + Ac*x18 + H*x2 + Hc*x6 + x21*x23 + x26*x28 - H*x4 - Hc*x8 - Pcj*x32 - x11*x26 - x16*x21 - x35*x50 - P0*U*x30 - Pc0*x33*x51 + (T(2.0)*(x33*x35*z));
  o.tI = (-dP0*(x52 + x40*z - Hc*z2)) - dPc0*(x53 + x46*z3 - H*z2) - dPcj*(x54 + x26*z2 + x32*z - A*z2) - dPj*(x55 + x21*z2 + x35*z3 - Ac*z2) - dQcj*x20*(x32 - x24) - dQj*x25*(x36 - x29);
  o.fII = (-x1) + x60*z2 - F*x57 - x58*x59 + U*x61*x62 + iU*x63*x64*z2;
  o.dII[0] = x65 - x59 + Pcj*z2;
  o.dII[1] = x66 - x57;
  o.dII[2] = x50 + x67 - F*z;
  o.dII[3] = x68 - x58*z;
  o.dII[4] = x61*x62 - x48*x63*x64;
  o.dII[5] = (-x49) - F*x56 - Fc*x58 - P0*x66 - Pc0*x68 - Pcj*x67 + (T(2.0)*(x60*z)) + F*Pc0*z + Fc*P0*z - iU*x50*x64 + (T(2.0)*(iU*x63*x64*z));
  o.tII = (-dP0*(x52 + x66*z - Fc*z2)) - dPc0*(x53 + x63*x69 - F*z2) - dPcj*(x54 + x67*z - B*z2) - dPj*(x55 + x64*x69 - Bc*z2);
  o.fIII = x71*x74 + x87*x88 + x90*x91 - x85*z - x90*x92;
  o.dIII[0] = x93*(x38 + x38*x78);
  o.dIII[1] = (-x92*x96) - e1*x62*x94 - x103*x75*(e1*e1) + U*e1*x62*x87 + iU*x84*x96*z2;
  o.dIII[2] = x105*x92 - e2*x104 - x105*x91 + e2*x31*x94 + x77*(e2*e2)*((-x104) - x33*x91 + x31*x84*z + x33*x87*z);
  o.dIII[3] = x74 + e1*x101 + x106*x95 - e1*x99 - x102*x95;
  o.dIII[4] = x76*(x98 - x107 + e1*x103);
  o.dIII[5] = (-x74) - e2*x108 - x106*x89 + e2*x100*x45*z + e2*x31*x97*z;
  o.dIII[6] = x78*(x107 - x98 - e2*(x108 + x47*x97 - x102*x45 - x31*x98));
  o.dIII[7] = x110*(x43 + x43*x83);
  o.dIII[8] = (-x125) - x118*(ec1*ec1) - x120*x122 + x120*x123*z;
  o.dIII[9] = x109*x126 - ec2*x127 - x126*x88 + x82*(ec2*ec2)*((-x127) - x30*x88 + x30*x90*z + x34*x79*z) + ec2*x34*x79*z;
  o.dIII[10] = x125 + x128 - x119*x129 + ec1*x121*x66;
  o.dIII[11] = ec1*(ec1*x118 + x124*x80 - x123*x51*x80);
  o.dIII[12] = (-x128) - ec2*x130 - ec2*x131 + ec2*x121*x34*z + ec2*x123*x39*z;
  o.dIII[13] = x83*((-x124) - ec2*(x130 + x131 - x124*x34 - x129*x39) + iU*x123*z2);
  o.dIII[14] = x100*x121 - x123*x48*x97;
  o.dIII[15] = (-x85) + x71*x73 - x87*x90 - P0*x132*x136 - Pc0*x133*x137 - x11*x134*x90 - x135*x16*x87 + P0*x132*x84*z + Pc0*x133*x79*z + Pcj*U*x134*x79 + (T(2.0)*(iU*x84*x90*z)) + Pj*iU*x135*x84*z2;
  o.tIII = dQcj*x110*(x20 + x20*x83) + dQj*x93*(x25 + x25*x78) + dP0*x132*z*((-x136) + x84*z) + dPc0*x133*z*((-x137) + x79*z) - dPcj*z*(x122 - x129)*(ec1*x113 + ec2*x82) - dPj*z*(x106 - x102)*(x116 - x111);
}

// The three equations alone: 62 complex mul, 57 complex add/sub, 0 real x complex.
#define FRG_GENF_CMUL 62
#define FRG_GENF_CADD 57
template <typename T>
__device__ __forceinline__ void frg_group_f(
    const cx<T> A, const cx<T> B, const cx<T> C, const cx<T> D, const cx<T> F, const cx<T> G,
    const cx<T> H, const cx<T> Ac, const cx<T> Bc, const cx<T> Cc, const cx<T> Dc, const cx<T> Fc,
    const cx<T> Gc, const cx<T> Hc, const cx<T> z,
    const cx<T> e1, const cx<T> e2, const cx<T> ec1, const cx<T> ec2,
    const cx<T> z2, const cx<T> z3, const cx<T> P0, const cx<T> Pc0,
    const cx<T> U, const cx<T> iU, const cx<T> Pj, const cx<T> Pcj, const cx<T> Qj, const cx<T> Qcj,
    cx<T>& fI, cx<T>& fII, cx<T>& fIII) {
  const cx<T> y0 = z3*(P0*Pc0 + Pcj*Pj);
  const cx<T> y1 = (-(Pc0*z));
  const cx<T> y2 = (-(P0*z));
  const cx<T> y3 = (-(Ac));
  const cx<T> y4 = Pcj*z;
  const cx<T> y5 = y3 + y4;
  const cx<T> y6 = (-(A));
  const cx<T> y7 = Pj*z;
  const cx<T> y8 = y6 + y7;
  const cx<T> y9 = (-(y7));
  const cx<T> y10 = A + y9;
  const cx<T> y11 = Ac - Cc;
  const cx<T> y12 = Qcj*y11;
  const cx<T> y13 = (-(y4));
  const cx<T> y14 = Ac + y13;
  const cx<T> y15 = A - C;
  const cx<T> y16 = Qj*y15;
  const cx<T> y17 = H + y2;
  const cx<T> y18 = Hc + y1;
  const cx<T> y19 = iU*z2;
  const cx<T> y20 = Bc + y13;
  const cx<T> y21 = F + y2;
  const cx<T> y22 = B + y9;
  const cx<T> y23 = Fc + y1;
  const cx<T> y24 = (-(G));
  const cx<T> y25 = (-(Gc));
  const cx<T> y26 = e1*(B - D);
  const cx<T> y27 = e2*(C + y24);
  const cx<T> y28 = y21*y26 - y17*y27;
  const cx<T> y29 = ec1*(Bc - Dc);
  const cx<T> y30 = ec2*(Cc + y25);
  const cx<T> y31 = y23*y29 - y18*y30;
  const cx<T> y32 = Bc + y12 + y3 + y20*y29 - y30*(y14 - Qcj*y11);
  const cx<T> y33 = B + y16 + y6 + y22*y26 - y27*(y10 - Qj*y15);
  fI = (-y0) + A*z*(Cc + y5) + Ac*z*(C + y8) + U*y17*((-y12) - y5) + y10*y12*z + y14*y16*z + y18*y19*((-y16) - y8) - H*z*(Cc + y1) - Hc*z*(C + y2);
  fII = (-y0) + z2*(B*Pcj + Bc*Pj) + U*y20*y21 - F*z*(Bc + y1) - Fc*z*(B + y2) + iU*y22*y23*z2;
  fIII = U*y28*y32 + y19*y31*y33 + z*(D + y24)*(Dc + y25) - y28*y31*z - y32*y33*z;
}
