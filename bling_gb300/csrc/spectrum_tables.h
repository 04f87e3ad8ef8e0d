/* Generated by bling_gb300/gen_spectrum_tables.py from bling's Spectrum.hs.
 * 16-band values as GHC computes them at start-up (fromSpd/avgSpd,
 * Spectrum.hs:297-335); bit patterns are exact binary32. Do not edit. */
#pragma once
#include <stdint.h>
#include <string.h>
#ifndef BLING_HD
#if defined(__CUDACC__)
#define BLING_HD __host__ __device__
#else
#define BLING_HD
#endif
#endif
static inline BLING_HD float __bling_f32(uint32_t b) { float f; memcpy(&f, &b, 4); return f; }
#define BLING_SPECTRUM_BANDS 16
/* index order of the RGB basis tables below */
enum { BLING_BASIS_WHITE, BLING_BASIS_CYAN, BLING_BASIS_MAGENTA, BLING_BASIS_YELLOW,
       BLING_BASIS_RED, BLING_BASIS_GREEN, BLING_BASIS_BLUE };

/* bit patterns, so the tables can live in __constant__ or host memory alike */
static const uint32_t BLING_CIE_X_BITS[16] = {
   0x3d3f2fadu, 0x3e75c9deu, 0x3ead7e3au, 0x3e73c70au,
   0x3d8c2d86u, 0x3bf6ec08u, 0x3dab3203u, 0x3e99b09eu,
   0x3f165bc6u, 0x3f61d673u, 0x3f85c8c7u, 0x3f6aee7au,
   0x3f0e6b6fu, 0x3e7a6cd8u, 0x3da8230eu, 0x3cc4b9b6u,
};
static const uint32_t BLING_CIE_Y_BITS[16] = {
   0x3aab8f57u, 0x3c23864eu, 0x3d0789e2u, 0x3d9f0613u,
   0x3e2f49d8u, 0x3ec2ef5eu, 0x3f39ccbeu, 0x3f72e162u,
   0x3f7d195bu, 0x3f6254c0u, 0x3f2ccb5au, 0x3edf3de8u,
   0x3e67253du, 0x3dbc91e5u, 0x3cf6518fu, 0x3c0e74ddu,
};
static const uint32_t BLING_CIE_Z_BITS[16] = {
   0x3e643667u, 0x3f95ff41u, 0x3fe0fd9bu, 0x3fba575eu,
   0x3f298be1u, 0x3e77cbc5u, 0x3d9f422au, 0x3cadd40eu,
   0x3b9550cau, 0x3ae02b27u, 0x3a6fb625u, 0x398a7d9eu,
   0x3826838cu, 0x36058befu, 0x00000000u, 0x00000000u,
};
#define BLING_CIE_Y_SUM_BITS 0x40b60abcu /* 5.688810348510742 */
static const uint32_t BLING_RGB_REFL_BITS[112] = {
   0x3f87e6f3u, 0x3f87fa54u, 0x3f87fe96u, 0x3f87ff99u,
   0x3f87faa8u, 0x3f87de5bu, 0x3f87d80bu, 0x3f87efabu,
   0x3f87ffb2u, 0x3f87febdu, 0x3f87ff87u, 0x3f87ffc5u,
   0x3f87fc06u, 0x3f87f0e9u, 0x3f87b505u, 0x3f87b209u,
   0x3f836f91u, 0x3f83a1f5u, 0x3f85f94du, 0x3f84951eu,
   0x3f84eb3du, 0x3f86d3f4u, 0x3f86d24bu, 0x3f86dc79u,
   0x3f87112bu, 0x3f6878f8u, 0x3e87e440u, 0xbba709b7u,
   0xbb9e9d6fu, 0x3b6b363fu, 0x3c0828f5u, 0x3c187713u,
   0x3f7d5ca5u, 0x3f81666bu, 0x3f8180ffu, 0x3f80671cu,
   0x3f63fad4u, 0x3e5da57cu, 0x3b4ca24fu, 0xbaf7882fu,
   0x392ce8b8u, 0x3e9121f8u, 0x3f5c0430u, 0x3f7efec3u,
   0x3f790ef7u, 0x3f6a8badu, 0x3f76d353u, 0x3f6ab5dfu,
   0xbbb452c1u, 0xbb9f9500u, 0x3d172249u, 0x3e1dd58eu,
   0x3ebe0877u, 0x3f3c3a4du, 0x3f80d516u, 0x3f868e1au,
   0x3f869428u, 0x3f8697f9u, 0x3f869241u, 0x3f86994bu,
   0x3f86934cu, 0x3f868d20u, 0x3f866141u, 0x3f860085u,
   0x3df334f7u, 0x3d998a01u, 0x3c577ffbu, 0x3c3fa20au,
   0x3b8e6c4cu, 0xbbc8ade8u, 0xbc04b5bdu, 0xbbe63f75u,
   0x3b1bbff4u, 0x3e4f0d27u, 0x3f5d0291u, 0x3f7f29d3u,
   0x3f7eed16u, 0x3f7f422du, 0x3f7d264bu, 0x3f770818u,
   0xbc139106u, 0xbc234958u, 0xbc0a000cu, 0x3ce5d665u,
   0x3ecf20a3u, 0x3f67a89bu, 0x3f7fd15cu, 0x3f7fe42bu,
   0x3f7fcef7u, 0x3f5d1cffu, 0x3e997852u, 0x3a1d2a68u,
   0xbbbb0bc2u, 0xbc05e958u, 0xbc079983u, 0xba55ce98u,
   0x3f7e3f08u, 0x3f7eec03u, 0x3f7ffc2bu, 0x3f7e11e7u,
   0x3f475a35u, 0x3eafa139u, 0x3d54c3e5u, 0xb9944565u,
   0x3a2e0ed7u, 0x3ada4999u, 0x3b18c21eu, 0x3cc3621cu,
   0x3d338605u, 0x3d4b4c77u, 0x3d240dd4u, 0x3ca04ce3u,
};
static const uint32_t BLING_RGB_ILLUM_BITS[112] = {
   0x3f9401dfu, 0x3f93fdf5u, 0x3f941157u, 0x3f940a3au,
   0x3f940903u, 0x3f940aebu, 0x3f92b0a9u, 0x3f90bdbdu,
   0x3f8b7d8du, 0x3f83d862u, 0x3f754751u, 0x3f69bbe0u,
   0x3f65bca8u, 0x3f638781u, 0x3f612850u, 0x3f61066cu,
   0x3f90f160u, 0x3f9162e6u, 0x3f91715au, 0x3f916854u,
   0x3f9167f0u, 0x3f9162b8u, 0x3f91609au, 0x3f915129u,
   0x3f8fbf77u, 0x3f6050f9u, 0x3eab2bf8u, 0x3cc50aa4u,
   0xbc3ed08bu, 0xbc19fd82u, 0xbbf5fdf5u, 0xbbd58487u,
   0x3f8908e5u, 0x3f89d201u, 0x3f896665u, 0x3f89f5b1u,
   0x3f853a19u, 0x3f07df23u, 0x3cdfd574u, 0xba96028au,
   0xb90efa38u, 0x3dba6291u, 0x3f10dc25u, 0x3f82e0ccu,
   0x3f89c27au, 0x3f84b347u, 0x3f83bfbdu, 0x3f850348u,
   0x3ab6c561u, 0x37960a03u, 0xb90238bcu, 0x3ccb3635u,
   0x3f057f55u, 0x3f844109u, 0x3f84afc3u, 0x3f84b122u,
   0x3f84ab5au, 0x3f84ad8bu, 0x3f8496cbu, 0x3f75dfc0u,
   0x3f4a3631u, 0x3f2aca2du, 0x3f192c89u, 0x3f12c591u,
   0x3d6ba755u, 0x3d3fb6d8u, 0x3cb523ccu, 0x3adaba8eu,
   0x3987e205u, 0xb85705afu, 0xb8fd4953u, 0xb993b181u,
   0x3c5b2ec4u, 0x3e37d9f3u, 0x3f100f26u, 0x3f5f83bdu,
   0x3f79f368u, 0x3f7dc419u, 0x3f7c387fu, 0x3f7c1a93u,
   0x3c9007c3u, 0x3b201e93u, 0xbb020ac8u, 0x3c1752f3u,
   0x3ee56acfu, 0x3f837b45u, 0x3f838c36u, 0x3f83ac19u,
   0x3f84b08au, 0x3f813446u, 0x3ea4b325u, 0x3b3a2470u,
   0x3c36f134u, 0x3c19fcc3u, 0xbad3951du, 0x3c7c2d93u,
   0x3f86e8c9u, 0x3f873499u, 0x3f876df2u, 0x3f874e64u,
   0x3f86a6efu, 0x3ee93f5fu, 0xbacb7a21u, 0xbacb5f35u,
   0xb9ad2ba4u, 0xba103701u, 0xbabbf725u, 0x3c5c77a9u,
   0x3d75e12cu, 0x3e02aee3u, 0x3e208e41u, 0x3e28970du,
};
/* X, Y, Z of the CIE daylight components S0, S1, S2 (spdToXYZ) */
static const uint32_t BLING_CIE_S012_XYZ_BITS[9] = {
   0x42bfc5a8u, 0x42c7d4e6u, 0x42e78a8cu, 0x3fe118c9u,
   0x3fe73922u, 0x42025d30u, 0x3fff7b82u, 0x3f37173eu,
   0xc00cffbfu,
};
/* noisePerms' permutation of 0..255 (Texture.hs:395-413), as an
 * initializer list for host and device arrays */
#define BLING_NOISE_PERM_LIST \
   151, 160, 137, 91, 90, 15, 131, 13, 201, 95, 96, 53, 194, 233, 7, 225, \
   140, 36, 103, 30, 69, 142, 8, 99, 37, 240, 21, 10, 23, 190, 6, 148, \
   247, 120, 234, 75, 0, 26, 197, 62, 94, 252, 219, 203, 117, 35, 11, 32, \
   57, 177, 33, 88, 237, 149, 56, 87, 174, 20, 125, 136, 171, 168, 68, 175, \
   74, 165, 71, 134, 139, 48, 27, 166, 77, 146, 158, 231, 83, 111, 229, 122, \
   60, 211, 133, 230, 220, 105, 92, 41, 55, 46, 245, 40, 244, 102, 143, 54, \
   65, 25, 63, 161, 1, 216, 80, 73, 209, 76, 132, 187, 208, 89, 18, 169, \
   200, 196, 135, 130, 116, 188, 159, 86, 164, 100, 109, 198, 173, 186, 3, 64, \
   52, 217, 226, 250, 124, 123, 5, 202, 38, 147, 118, 126, 255, 82, 85, 212, \
   207, 206, 59, 227, 47, 16, 58, 17, 182, 189, 28, 42, 223, 183, 170, 213, \
   119, 248, 152, 2, 44, 154, 163, 70, 221, 153, 101, 155, 167, 43, 172, 9, \
   129, 22, 39, 253, 19, 98, 108, 110, 79, 113, 224, 232, 178, 185, 112, 104, \
   218, 246, 97, 228, 251, 34, 242, 193, 238, 210, 144, 12, 191, 179, 162, 241, \
   81, 51, 145, 235, 249, 14, 239, 107, 49, 192, 214, 31, 181, 199, 106, 157, \
   184, 84, 204, 176, 115, 121, 50, 45, 127, 4, 150, 254, 138, 236, 205, 93, \
   222, 114, 67, 29, 24, 72, 243, 141, 128, 195, 78, 66, 215, 61, 156, 180

