/*
 * oxDNA2 model constants.
 *
 * Values are those of the reference model definition (src/model.h:11-436 and
 * src/defs.h:14).  Every value there is a float literal, so code computing in double sees
 * the float-rounded value, exactly as the reference's double-precision build does; the
 * literals below keep the `f` suffix for that reason, and composite values (theta0 = pi - x,
 * ...) are written as float expressions for the same reason.
 *
 * Plain C preprocessor header: included by the CUDA kernels, by the host parameter builder
 * and by the CPU oracle.
 */
#ifndef OXGB_DNA2_MODEL_H
#define OXGB_DNA2_MODEL_H

#define OXM_PI 3.141592653589793238462643f /* src/defs.h:14 (a float) */

/* interaction-site offsets along the body axes a1 (and a2 for the grooved backbone),
 * src/model.h:11-18; GAMMA = POS_STACK - POS_BACK (src/model.h:41) */
#define OXM_POS_BACK -0.4f
#define OXM_POS_MM_BACK1 -0.3400f
#define OXM_POS_MM_BACK2 0.3408f
#define OXM_POS_STACK 0.34f
#define OXM_POS_BASE 0.4f
#define OXM_GAMMA 0.74f

/* FENE backbone, src/model.h:46-52 */
#define OXM_FENE_EPS 2.0f
#define OXM_FENE_R0_OXDNA 0.7525f
#define OXM_FENE_R0_OXDNA2 0.7564f
#define OXM_FENE_DELTA 0.25f
#define OXM_FENE_DELTA2 0.0625f

/* excluded volume; site pairs 1 = back-back, 2 = base-base, 3 = base(p)-back(q),
 * 4 = back(p)-base(q); src/model.h:56-84 */
#define OXM_EXCL_EPS 2.0f
#define OXM_EXCL_S1 0.70f
#define OXM_EXCL_S2 0.33f
#define OXM_EXCL_S3 0.515f
#define OXM_EXCL_S4 0.515f
#define OXM_EXCL_R1 0.675f
#define OXM_EXCL_R2 0.32f
#define OXM_EXCL_R3 0.50f
#define OXM_EXCL_R4 0.50f
#define OXM_EXCL_B1 892.016223343f
#define OXM_EXCL_B2 4119.70450017f
#define OXM_EXCL_B3 1707.30627298f
#define OXM_EXCL_B4 1707.30627298f
#define OXM_EXCL_RC1 0.711879214356f
#define OXM_EXCL_RC2 0.335388426126f
#define OXM_EXCL_RC3 0.52329943261f
#define OXM_EXCL_RC4 0.52329943261f

/* radial Morse f1: index 0 = hydrogen bonding, 1 = stacking; src/model.h:91-105,152-166 */
#define OXM_F1_HB 0
#define OXM_F1_ST 1
#define OXM_HYDR_EPS_OXDNA 1.077f
#define OXM_HYDR_EPS_OXDNA2 1.0678f
#define OXM_STCK_BASE_EPS_OXDNA 1.3448f
#define OXM_STCK_FACT_EPS_OXDNA 2.6568f
#define OXM_STCK_BASE_EPS_OXDNA2 1.3523f
#define OXM_STCK_FACT_EPS_OXDNA2 2.6717f
#define OXM_F1_TABLE_A {8.f, 6.f}
#define OXM_F1_TABLE_RC {0.75f, 0.9f}
#define OXM_F1_TABLE_R0 {0.4f, 0.4f}
#define OXM_F1_TABLE_BLOW {-126.243f, -68.1857f}
#define OXM_F1_TABLE_BHIGH {-7.87708f, -3.12992f}
#define OXM_F1_TABLE_RLOW {0.34f, 0.32f}
#define OXM_F1_TABLE_RHIGH {0.7f, 0.75f}
#define OXM_F1_TABLE_RCLOW {0.276908f, 0.23239f}
#define OXM_F1_TABLE_RCHIGH {0.783775f, 0.956f}
#define OXM_HYDR_RCLOW 0.276908f
#define OXM_HYDR_RCHIGH 0.783775f

/* radial harmonic f2: index 0 = cross stacking, 1 = coaxial stacking; src/model.h:210-219,
 * 330-341.  The coaxial K is the oxDNA2 value (src/Interactions/DNA2Interaction.cpp:9). */
#define OXM_F2_CRST 0
#define OXM_F2_CXST 1
#define OXM_CXST_K_OXDNA 46.0f
#define OXM_CXST_K_OXDNA2 58.5f
#define OXM_F2_TABLE_K {47.5f, 58.5f}
#define OXM_F2_TABLE_RC {0.675f, 0.6f}
#define OXM_F2_TABLE_R0 {0.575f, 0.400f}
#define OXM_F2_TABLE_BLOW {-0.888889f, -2.13158f}
#define OXM_F2_TABLE_RLOW {0.495f, 0.22f}
#define OXM_F2_TABLE_RCLOW {0.45f, 0.177778f}
#define OXM_F2_TABLE_BHIGH {-0.888889f, -2.13158f}
#define OXM_F2_TABLE_RHIGH {0.655f, 0.58f}
#define OXM_F2_TABLE_RCHIGH {0.7f, 0.6222222f}
#define OXM_CRST_RCLOW 0.45f
#define OXM_CRST_RCHIGH 0.7f
#define OXM_CXST_RCLOW 0.177778f
#define OXM_CXST_RCHIGH 0.6222222f

/* angular modulation f4(theta) = 1 - A (theta - T0)^2 inside TS, B (TC - |theta - T0|)^2
 * up to TC, zero beyond; thirteen parameter sets, numbered as in the reference
 * (src/model.h: *_F4_THETA* indices and *_THETA*_{A,B,T0,TS,TC}).  Set 10 carries the
 * oxDNA2 coaxial theta1 centre and its extra pure-harmonic term (SA, SB). */
#define OXM_F4_ST_T4 0
#define OXM_F4_ST_T5 1 /* also theta6 */
#define OXM_F4_HB_T1 2
#define OXM_F4_HB_T2 3 /* also theta3 */
#define OXM_F4_HB_T4 4
#define OXM_F4_HB_T7 5 /* also theta8 */
#define OXM_F4_CR_T1 6
#define OXM_F4_CR_T2 7 /* also theta3 */
#define OXM_F4_CR_T4 8
#define OXM_F4_CR_T7 9 /* also theta8 */
#define OXM_F4_CX_T1 10
#define OXM_F4_CX_T4 11
#define OXM_F4_CX_T5 12 /* also theta6 */
#define OXM_N_F4 13

#define OXM_F4_TABLE_A {1.3f, 0.9f, 1.5f, 1.5f, 0.46f, 4.f, 2.25f, 1.70f, 1.50f, 1.70f, 2.f, 1.3f, 0.9f}
#define OXM_F4_TABLE_B \
	{6.4381f, 3.89361f, 4.16038f, 4.16038f, 0.133855f, 17.0526f, 7.00545f, 6.2469f, 2.59556f, 6.2469f, 10.9032f, 6.4381f, 3.89361f}
#define OXM_F4_TABLE_T0 \
	{0.f, 0.f, 0.f, 0.f, OXM_PI, (OXM_PI * 0.5f), (OXM_PI - 2.35f), 1.f, 0.f, 0.875f, (OXM_PI - 0.25f), 0.f, 0.f}
#define OXM_F4_TABLE_TS {0.8f, 0.95f, 0.7f, 0.7f, 0.7f, 0.45f, 0.58f, 0.68f, 0.65f, 0.68f, 0.65f, 0.8f, 0.95f}
#define OXM_F4_TABLE_TC \
	{0.961538f, 1.16959f, 0.952381f, 0.952381f, 3.10559f, 0.555556f, 0.766284f, 0.865052f, 1.02564f, 0.865052f, 0.769231f, 0.961538f, 1.16959f}
/* oxDNA2 coaxial theta1 extra harmonic: f = SA (theta - SB)^2 for theta > SB */
#define OXM_CXST_THETA1_SA 20.f
#define OXM_CXST_THETA1_SB (OXM_PI - 0.1f * (OXM_PI - (OXM_PI - 0.25f)))

/* cos(phi) modulation f5: 0 = stacking phi1, 1 = stacking phi2, 2 = coaxial phi3,
 * 3 = coaxial phi4 (the reference stores PHI3_B in slot 3); src/model.h:184-193,380-389 */
#define OXM_F5_PHI1 0
#define OXM_F5_PHI2 1
#define OXM_F5_TABLE_A {2.0f, 2.0f, 2.0f, 2.0f}
#define OXM_F5_TABLE_B {10.9032f, 10.9032f, 10.9032f, 10.9032f}
#define OXM_F5_TABLE_XC {-0.769231f, -0.769231f, -0.769231f, -0.769231f}
#define OXM_F5_TABLE_XS {-0.65f, -0.65f, -0.65f, -0.65f}

/* Debye-Hueckel defaults: lambda at T = 300 K and I = 1 M, and the prefactor
 * (src/Interactions/DNA2Interaction.cpp:74-81) */
#define OXM_DH_LAMBDA_DEFAULT 0.3616455
#define OXM_DH_STRENGTH_DEFAULT 0.0543

/* base codes: A = 0, G = 1, C = 2, T = 3 (Watson-Crick partners sum to 3), 4 = dummy */
#define OXM_N_BASE_TYPES 5

#endif
