/*
 * metric_ref_shim.h -- TEST INFRASTRUCTURE ONLY.  Declarations that let the
 * reference's geometry routines build on their own for the parity pin of
 * the geometry producer: metric_term() (Grid_Transformation.cpp, compiled
 * where it lies) and the half-point block of Main.cpp:2369-2440 (cut out of
 * Main.cpp by build_ref.sh into oracle/_ref/ and wrapped in a function).
 * The types keep the reference's field layout (functions.h:22-36, 93-135,
 * the parts these routines read); the globals are defined in
 * ref_metrics.cpp.  No MPI or OpenCL header is involved.
 */
#pragma once

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>

using std::cin;
using std::cout;
using std::ifstream;
using std::istringstream;
using std::ofstream;
using std::string;
using std::stringstream;
using std::vector;

typedef struct {
    double x, y, z;
    int e[8];
    int ID;
    int n_n[7];
    int corner_ID;
    int val;
    int loc;
    int proc;
    int local;
    int global;
    int req;
} MNODE;

typedef struct {
    double x_zeta, x_eta, x_xi, y_zeta, y_eta, y_xi, z_zeta, z_eta, z_xi;
} JACOB;

typedef struct {
    double zeta_1, zeta_2, zeta_3;
    double eta_1, eta_2, eta_3;
    double xi_1, xi_2, xi_3;
} JAC;

typedef struct {
    double zeta_1, zeta_2, zeta_3, zeta_4, zeta_5, zeta_6;
    double eta_1, eta_2, eta_3, eta_4, eta_5, eta_6;
    double xi_1, xi_2, xi_3, xi_4, xi_5, xi_6;
} TEMP_JAC;

typedef struct {
    int connect[9], element_neighbour[9];
    int type;
    int location;
    int corner;
} ELEM;

typedef struct __attribute__((packed)) {
    double zeta_x, zeta_y, zeta_z, eta_x, eta_y, eta_z, xi_x, xi_y, xi_z;
    double zeta_xip, zeta_yip, zeta_zip, eta_xip, eta_yip, eta_zip, xi_xip, xi_yip, xi_zip, zeta_xim, zeta_yim,
        zeta_zim, eta_xim, eta_yim, eta_zim, xi_xim, xi_yim, xi_zim;
    double zeta_xjp, zeta_yjp, zeta_zjp, eta_xjp, eta_yjp, eta_zjp, xi_xjp, xi_yjp, xi_zjp, zeta_xjm, zeta_yjm,
        zeta_zjm, eta_xjm, eta_yjm, eta_zjm, xi_xjm, xi_yjm, xi_zjm;
    double zeta_xkp, zeta_ykp, zeta_zkp, eta_xkp, eta_ykp, eta_zkp, xi_xkp, xi_ykp, xi_zkp, zeta_xkm, zeta_ykm,
        zeta_zkm, eta_xkm, eta_ykm, eta_zkm, xi_xkm, xi_ykm, xi_zkm;
} TRANSFORMED;

typedef struct __attribute__((packed)) {
    double ip, im, jp, jm, kp, km;
} DETERM;

extern vector<MNODE> node;
extern vector<JACOB> jacobian;
extern vector<JAC> jac;
extern vector<TEMP_JAC> jaco;
extern vector<ELEM> CD;
extern vector<TRANSFORMED> metric;
extern vector<DETERM> deter;
extern vector<double> det;
extern vector<int> all_boundary_nodes;
extern int all_bou_node, NUMNP, h, i, sd_node;
extern double del_zeta, del_eta;

void metric_term();
void ref_half_points_body();
