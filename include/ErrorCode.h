/*
 * ErrorCode.h -- OpenCUDA's error codes (okano_3_0/ErrorCode.h:16-56), kept
 * with the same names and values so callers of the reference compile and
 * branch unchanged.
 */
#ifndef __ERRORCODE_H__
#define __ERRORCODE_H__

#define NO_ERROR        0
#define INVALID_DATA   -1
#define NULL_POINTER   -2
#define OP_OVERFLOW    -3
#define NO_FILE        -4
#define WRONG_FILE     -5
#define OUT_OF_MEM     -6
#define CUDA_ERROR     -7
#define UNMATCH_IMG    -8
#define UNIMPLEMENT  -998
#define UNKNOW_ERROR -999

#endif
