// Generated by gen_twiddles.py: c_tw<R>[m] = (cos(2 pi m/R), sin(2 pi m/R)), m < R.
#pragma once
#include <cuda_runtime.h>

namespace mrsr {

static __constant__ float2 c_tw32[32] = {
    {0x1.0000000000000p+0f, 0x0.0p+0f}, {0x1.f6297c0000000p-1f, 0x1.8f8b840000000p-3f}, {0x1.d906bc0000000p-1f, 0x1.87de2a0000000p-2f}, {0x1.a9b6620000000p-1f, 0x1.1c73b40000000p-1f},
    {0x1.6a09e60000000p-1f, 0x1.6a09e60000000p-1f}, {0x1.1c73b40000000p-1f, 0x1.a9b6620000000p-1f}, {0x1.87de2a0000000p-2f, 0x1.d906bc0000000p-1f}, {0x1.8f8b840000000p-3f, 0x1.f6297c0000000p-1f},
    {0x0.0p+0f, 0x1.0000000000000p+0f}, {-0x1.8f8b840000000p-3f, 0x1.f6297c0000000p-1f}, {-0x1.87de2a0000000p-2f, 0x1.d906bc0000000p-1f}, {-0x1.1c73b40000000p-1f, 0x1.a9b6620000000p-1f},
    {-0x1.6a09e60000000p-1f, 0x1.6a09e60000000p-1f}, {-0x1.a9b6620000000p-1f, 0x1.1c73b40000000p-1f}, {-0x1.d906bc0000000p-1f, 0x1.87de2a0000000p-2f}, {-0x1.f6297c0000000p-1f, 0x1.8f8b840000000p-3f},
    {-0x1.0000000000000p+0f, 0x0.0p+0f}, {-0x1.f6297c0000000p-1f, -0x1.8f8b840000000p-3f}, {-0x1.d906bc0000000p-1f, -0x1.87de2a0000000p-2f}, {-0x1.a9b6620000000p-1f, -0x1.1c73b40000000p-1f},
    {-0x1.6a09e60000000p-1f, -0x1.6a09e60000000p-1f}, {-0x1.1c73b40000000p-1f, -0x1.a9b6620000000p-1f}, {-0x1.87de2a0000000p-2f, -0x1.d906bc0000000p-1f}, {-0x1.8f8b840000000p-3f, -0x1.f6297c0000000p-1f},
    {0x0.0p+0f, -0x1.0000000000000p+0f}, {0x1.8f8b840000000p-3f, -0x1.f6297c0000000p-1f}, {0x1.87de2a0000000p-2f, -0x1.d906bc0000000p-1f}, {0x1.1c73b40000000p-1f, -0x1.a9b6620000000p-1f},
    {0x1.6a09e60000000p-1f, -0x1.6a09e60000000p-1f}, {0x1.a9b6620000000p-1f, -0x1.1c73b40000000p-1f}, {0x1.d906bc0000000p-1f, -0x1.87de2a0000000p-2f}, {0x1.f6297c0000000p-1f, -0x1.8f8b840000000p-3f},
};

static __constant__ float2 c_tw24[24] = {
    {0x1.0000000000000p+0f, 0x0.0p+0f}, {0x1.ee8dd40000000p-1f, 0x1.0907dc0000000p-2f}, {0x1.bb67ae0000000p-1f, 0x1.0000000000000p-1f}, {0x1.6a09e60000000p-1f, 0x1.6a09e60000000p-1f},
    {0x1.0000000000000p-1f, 0x1.bb67ae0000000p-1f}, {0x1.0907dc0000000p-2f, 0x1.ee8dd40000000p-1f}, {0x0.0p+0f, 0x1.0000000000000p+0f}, {-0x1.0907dc0000000p-2f, 0x1.ee8dd40000000p-1f},
    {-0x1.0000000000000p-1f, 0x1.bb67ae0000000p-1f}, {-0x1.6a09e60000000p-1f, 0x1.6a09e60000000p-1f}, {-0x1.bb67ae0000000p-1f, 0x1.0000000000000p-1f}, {-0x1.ee8dd40000000p-1f, 0x1.0907dc0000000p-2f},
    {-0x1.0000000000000p+0f, 0x0.0p+0f}, {-0x1.ee8dd40000000p-1f, -0x1.0907dc0000000p-2f}, {-0x1.bb67ae0000000p-1f, -0x1.0000000000000p-1f}, {-0x1.6a09e60000000p-1f, -0x1.6a09e60000000p-1f},
    {-0x1.0000000000000p-1f, -0x1.bb67ae0000000p-1f}, {-0x1.0907dc0000000p-2f, -0x1.ee8dd40000000p-1f}, {0x0.0p+0f, -0x1.0000000000000p+0f}, {0x1.0907dc0000000p-2f, -0x1.ee8dd40000000p-1f},
    {0x1.0000000000000p-1f, -0x1.bb67ae0000000p-1f}, {0x1.6a09e60000000p-1f, -0x1.6a09e60000000p-1f}, {0x1.bb67ae0000000p-1f, -0x1.0000000000000p-1f}, {0x1.ee8dd40000000p-1f, -0x1.0907dc0000000p-2f},
};

static __constant__ float2 c_tw20[20] = {
    {0x1.0000000000000p+0f, 0x0.0p+0f}, {0x1.e6f0e20000000p-1f, 0x1.3c6ef40000000p-2f}, {0x1.9e377a0000000p-1f, 0x1.2cf2300000000p-1f}, {0x1.2cf2300000000p-1f, 0x1.9e377a0000000p-1f},
    {0x1.3c6ef40000000p-2f, 0x1.e6f0e20000000p-1f}, {0x0.0p+0f, 0x1.0000000000000p+0f}, {-0x1.3c6ef40000000p-2f, 0x1.e6f0e20000000p-1f}, {-0x1.2cf2300000000p-1f, 0x1.9e377a0000000p-1f},
    {-0x1.9e377a0000000p-1f, 0x1.2cf2300000000p-1f}, {-0x1.e6f0e20000000p-1f, 0x1.3c6ef40000000p-2f}, {-0x1.0000000000000p+0f, 0x0.0p+0f}, {-0x1.e6f0e20000000p-1f, -0x1.3c6ef40000000p-2f},
    {-0x1.9e377a0000000p-1f, -0x1.2cf2300000000p-1f}, {-0x1.2cf2300000000p-1f, -0x1.9e377a0000000p-1f}, {-0x1.3c6ef40000000p-2f, -0x1.e6f0e20000000p-1f}, {0x0.0p+0f, -0x1.0000000000000p+0f},
    {0x1.3c6ef40000000p-2f, -0x1.e6f0e20000000p-1f}, {0x1.2cf2300000000p-1f, -0x1.9e377a0000000p-1f}, {0x1.9e377a0000000p-1f, -0x1.2cf2300000000p-1f}, {0x1.e6f0e20000000p-1f, -0x1.3c6ef40000000p-2f},
};

static __constant__ float2 c_tw30[30] = {
    {0x1.0000000000000p+0f, 0x0.0p+0f}, {0x1.f4cfc40000000p-1f, 0x1.a9cd9a0000000p-3f}, {0x1.d3bc3a0000000p-1f, 0x1.a07f920000000p-2f}, {0x1.9e377a0000000p-1f, 0x1.2cf2300000000p-1f},
    {0x1.56984a0000000p-1f, 0x1.7c7d7a0000000p-1f}, {0x1.0000000000000p-1f, 0x1.bb67ae0000000p-1f}, {0x1.3c6ef40000000p-2f, 0x1.e6f0e20000000p-1f}, {0x1.ac260a0000000p-4f, 0x1.fd31fa0000000p-1f},
    {-0x1.ac260a0000000p-4f, 0x1.fd31fa0000000p-1f}, {-0x1.3c6ef40000000p-2f, 0x1.e6f0e20000000p-1f}, {-0x1.0000000000000p-1f, 0x1.bb67ae0000000p-1f}, {-0x1.56984a0000000p-1f, 0x1.7c7d7a0000000p-1f},
    {-0x1.9e377a0000000p-1f, 0x1.2cf2300000000p-1f}, {-0x1.d3bc3a0000000p-1f, 0x1.a07f920000000p-2f}, {-0x1.f4cfc40000000p-1f, 0x1.a9cd9a0000000p-3f}, {-0x1.0000000000000p+0f, 0x0.0p+0f},
    {-0x1.f4cfc40000000p-1f, -0x1.a9cd9a0000000p-3f}, {-0x1.d3bc3a0000000p-1f, -0x1.a07f920000000p-2f}, {-0x1.9e377a0000000p-1f, -0x1.2cf2300000000p-1f}, {-0x1.56984a0000000p-1f, -0x1.7c7d7a0000000p-1f},
    {-0x1.0000000000000p-1f, -0x1.bb67ae0000000p-1f}, {-0x1.3c6ef40000000p-2f, -0x1.e6f0e20000000p-1f}, {-0x1.ac260a0000000p-4f, -0x1.fd31fa0000000p-1f}, {0x1.ac260a0000000p-4f, -0x1.fd31fa0000000p-1f},
    {0x1.3c6ef40000000p-2f, -0x1.e6f0e20000000p-1f}, {0x1.0000000000000p-1f, -0x1.bb67ae0000000p-1f}, {0x1.56984a0000000p-1f, -0x1.7c7d7a0000000p-1f}, {0x1.9e377a0000000p-1f, -0x1.2cf2300000000p-1f},
    {0x1.d3bc3a0000000p-1f, -0x1.a07f920000000p-2f}, {0x1.f4cfc40000000p-1f, -0x1.a9cd9a0000000p-3f},
};

// c_tw32 as broadcast half2 bit patterns: {(cos, cos), (sin, sin)}
static __constant__ unsigned int c_tw32_h2[32][2] = {
    {0x3c003c00u, 0x00000000u}, {0x3bd93bd9u, 0x323e323eu}, {0x3b643b64u, 0x361f361fu}, {0x3aa73aa7u, 0x38723872u},
    {0x39a839a8u, 0x39a839a8u}, {0x38723872u, 0x3aa73aa7u}, {0x361f361fu, 0x3b643b64u}, {0x323e323eu, 0x3bd93bd9u},
    {0x00000000u, 0x3c003c00u}, {0xb23eb23eu, 0x3bd93bd9u}, {0xb61fb61fu, 0x3b643b64u}, {0xb872b872u, 0x3aa73aa7u},
    {0xb9a8b9a8u, 0x39a839a8u}, {0xbaa7baa7u, 0x38723872u}, {0xbb64bb64u, 0x361f361fu}, {0xbbd9bbd9u, 0x323e323eu},
    {0xbc00bc00u, 0x00000000u}, {0xbbd9bbd9u, 0xb23eb23eu}, {0xbb64bb64u, 0xb61fb61fu}, {0xbaa7baa7u, 0xb872b872u},
    {0xb9a8b9a8u, 0xb9a8b9a8u}, {0xb872b872u, 0xbaa7baa7u}, {0xb61fb61fu, 0xbb64bb64u}, {0xb23eb23eu, 0xbbd9bbd9u},
    {0x00000000u, 0xbc00bc00u}, {0x323e323eu, 0xbbd9bbd9u}, {0x361f361fu, 0xbb64bb64u}, {0x38723872u, 0xbaa7baa7u},
    {0x39a839a8u, 0xb9a8b9a8u}, {0x3aa73aa7u, 0xb872b872u}, {0x3b643b64u, 0xb61fb61fu}, {0x3bd93bd9u, 0xb23eb23eu},
};

// c_tw24 as broadcast half2 bit patterns: {(cos, cos), (sin, sin)}
static __constant__ unsigned int c_tw24_h2[24][2] = {
    {0x3c003c00u, 0x00000000u}, {0x3bba3bbau, 0x34243424u}, {0x3aee3aeeu, 0x38003800u}, {0x39a839a8u, 0x39a839a8u},
    {0x38003800u, 0x3aee3aeeu}, {0x34243424u, 0x3bba3bbau}, {0x00000000u, 0x3c003c00u}, {0xb424b424u, 0x3bba3bbau},
    {0xb800b800u, 0x3aee3aeeu}, {0xb9a8b9a8u, 0x39a839a8u}, {0xbaeebaeeu, 0x38003800u}, {0xbbbabbbau, 0x34243424u},
    {0xbc00bc00u, 0x00000000u}, {0xbbbabbbau, 0xb424b424u}, {0xbaeebaeeu, 0xb800b800u}, {0xb9a8b9a8u, 0xb9a8b9a8u},
    {0xb800b800u, 0xbaeebaeeu}, {0xb424b424u, 0xbbbabbbau}, {0x00000000u, 0xbc00bc00u}, {0x34243424u, 0xbbbabbbau},
    {0x38003800u, 0xbaeebaeeu}, {0x39a839a8u, 0xb9a8b9a8u}, {0x3aee3aeeu, 0xb800b800u}, {0x3bba3bbau, 0xb424b424u},
};

// c_tw20 as broadcast half2 bit patterns: {(cos, cos), (sin, sin)}
static __constant__ unsigned int c_tw20_h2[20][2] = {
    {0x3c003c00u, 0x00000000u}, {0x3b9c3b9cu, 0x34f234f2u}, {0x3a793a79u, 0x38b438b4u}, {0x38b438b4u, 0x3a793a79u},
    {0x34f234f2u, 0x3b9c3b9cu}, {0x00000000u, 0x3c003c00u}, {0xb4f2b4f2u, 0x3b9c3b9cu}, {0xb8b4b8b4u, 0x3a793a79u},
    {0xba79ba79u, 0x38b438b4u}, {0xbb9cbb9cu, 0x34f234f2u}, {0xbc00bc00u, 0x00000000u}, {0xbb9cbb9cu, 0xb4f2b4f2u},
    {0xba79ba79u, 0xb8b4b8b4u}, {0xb8b4b8b4u, 0xba79ba79u}, {0xb4f2b4f2u, 0xbb9cbb9cu}, {0x00000000u, 0xbc00bc00u},
    {0x34f234f2u, 0xbb9cbb9cu}, {0x38b438b4u, 0xba79ba79u}, {0x3a793a79u, 0xb8b4b8b4u}, {0x3b9c3b9cu, 0xb4f2b4f2u},
};

// c_tw30 as broadcast half2 bit patterns: {(cos, cos), (sin, sin)}
static __constant__ unsigned int c_tw30_h2[30][2] = {
    {0x3c003c00u, 0x00000000u}, {0x3bd33bd3u, 0x32a732a7u}, {0x3b4f3b4fu, 0x36823682u}, {0x3a793a79u, 0x38b438b4u},
    {0x395a395au, 0x39f239f2u}, {0x38003800u, 0x3aee3aeeu}, {0x34f234f2u, 0x3b9c3b9cu}, {0x2eb12eb1u, 0x3bf53bf5u},
    {0xaeb1aeb1u, 0x3bf53bf5u}, {0xb4f2b4f2u, 0x3b9c3b9cu}, {0xb800b800u, 0x3aee3aeeu}, {0xb95ab95au, 0x39f239f2u},
    {0xba79ba79u, 0x38b438b4u}, {0xbb4fbb4fu, 0x36823682u}, {0xbbd3bbd3u, 0x32a732a7u}, {0xbc00bc00u, 0x00000000u},
    {0xbbd3bbd3u, 0xb2a7b2a7u}, {0xbb4fbb4fu, 0xb682b682u}, {0xba79ba79u, 0xb8b4b8b4u}, {0xb95ab95au, 0xb9f2b9f2u},
    {0xb800b800u, 0xbaeebaeeu}, {0xb4f2b4f2u, 0xbb9cbb9cu}, {0xaeb1aeb1u, 0xbbf5bbf5u}, {0x2eb12eb1u, 0xbbf5bbf5u},
    {0x34f234f2u, 0xbb9cbb9cu}, {0x38003800u, 0xbaeebaeeu}, {0x395a395au, 0xb9f2b9f2u}, {0x3a793a79u, 0xb8b4b8b4u},
    {0x3b4f3b4fu, 0xb682b682u}, {0x3bd33bd3u, 0xb2a7b2a7u},
};

}  // namespace mrsr
