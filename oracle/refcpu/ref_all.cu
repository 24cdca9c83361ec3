/*
 * One translation unit over the reference's own sources (found through -I
 * on the reference tree; nothing is copied), so that nvcc's host pass can
 * build the unmodified reference program without relocatable device code.
 * The list is the reference Makefile's (Makefile:7) minus helper.cu, whose
 * two used helpers ref_support.cpp provides, and hardCoded.cu, which is not
 * in the reference tree (ref_support.cpp defines the tables).
 *
 * Test infrastructure only (oracle/build_ref.sh).
 */
#include "mainPUMP.cu"
#include "obstacles.cu"
#include "sampler.cu"
#include "bvls.cu"
#include "hsmc.cu"
#include "collisionCheck.cu"
#include "2pBVP.cu"
#include "PUMP.cu"
#include "collisionProbability.cu"
#include "motionPlanningProblem.cu"
