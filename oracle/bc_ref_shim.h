/*
 * bc_ref_shim.h -- TEST INFRASTRUCTURE ONLY.  Declarations that let the
 * reference's boundary routine (Flow_Initialisation.cpp, compiled from the
 * copy build_ref.sh writes under oracle/_ref/) build on its own: the node,
 * singular-node and FLOW types with the reference's field layout
 * (functions.h:22-84, the parts the routine reads) and the globals it uses,
 * defined in ref_bc.cpp.  No MPI or OpenCL header is involved.
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
    int n_n[7];
} singul;

typedef struct __attribute__((packed)) {
    double u, v, w, p, t, rho, mu, a, e;
} FLOW_VARIABLES;

extern vector<MNODE> node;
extern vector<singul> singular;
extern vector<FLOW_VARIABLES> FLOW;
extern vector<int> inlet_node, outlet_node, wall_node, boundary_node;
extern vector<int> sd_inlet_node, sd_outlet_node, sd_wall_node, sd_boundary_node;
extern int out_node, inl_node, wal_node, bou_node, sd_out_node, sd_inl_node, sd_wal_node, sd_bou_node;
extern int initial, i, h, sd_node;
extern double Mach;

void intialise(int RK);
