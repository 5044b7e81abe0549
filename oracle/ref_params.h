/*
 * ref_params.h — force-included into every translation unit of the
 * reference build (oracle/_ref).  TEST INFRASTRUCTURE ONLY.
 *
 * The reference hard-codes the mEVP relaxation constants as class members
 * initialised to 1500 (dynamics/src/include/VPCGDynamicsKernel.hpp:125-126,
 * dynamics/src/include/MEVPStressUpdateStep.hpp:126-127).  The build recipe
 * (oracle/Makefile, target ref) writes copies of those two headers into
 * oracle/_ref/gen/ in which the literal is replaced by these two globals, so
 * one build serves alpha = beta = 300 (the box-test workload) and 1500 (the
 * reference default).  The harness sets them before it constructs a kernel;
 * the members read them at construction.
 */
#ifndef NSDG_REF_PARAMS_H
#define NSDG_REF_PARAMS_H
extern double nsdg_ref_alpha;
extern double nsdg_ref_beta;
#endif
