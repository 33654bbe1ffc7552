// Generated by fit_split_kernel.py -- do not edit.
// erfcx(u) ~= sum_k SPLIT_A[k] t^(k+1), t = 1/(1 + SPLIT_P u), u in [0, 4.0]
// max relative error of g(u) in double precision: 1.748e-07
#pragma once
#define SPLIT_NA 6
static const double SPLIT_P = 0.40999999999999998;
static const double SPLIT_A[SPLIT_NA] = {0.23491450949233103, 0.19206493278114967, 0.38580199800648118, -0.22375887226293992, 0.59516597649070491, -0.18418871825201483};
