/*
 * lpg_detmath.h — deterministic double-precision elementary functions.
 *
 * Every function here is built from IEEE-754 operations that are correctly
 * rounded on every target this project compiles for (add, sub, mul, div,
 * sqrt, floor, and exact power-of-two scaling), evaluated in a fixed order.
 * Compiled with contraction disabled (gcc -ffp-contract=off, nvcc
 * --fmad=false) the same input gives the same bits on x86-64, aarch64 and
 * sm_103a.  That is what lets the CUDA engine and the CPU oracle consume one
 * counter-based random stream and agree bit for bit on every integer draw
 * that depends on an exp() or a log() (Poisson counts, gamma variates,
 * probabilities of exposure).
 *
 * Methods (all textbook mathematics, table values computed here from
 * 60-digit decimal arithmetic by gen_detmath_tables.py, not taken from any
 * vendor library): table-driven reductions (Tang's method) that leave a
 * short polynomial, because double-precision latency, not throughput,
 * bounds the single-thread draws on the GPU (a dependent add or multiply
 * takes about 65 cycles on the GB300, a division about 430).
 *   exp    x = (64 q + j) ln2/64 + r with a two-part ln2/64 (the high part
 *          with 33 significant bits so k*hi is exact), |r| <= ln2/128;
 *          e^x = 2^q * 2^(j/64) * (1 + (e^r - 1)), 2^(j/64) a double-double
 *          from the table, e^r - 1 to degree 6, exact scaling by 2^q.
 *   expm1  the degree-6 series for |x| <= ln2/128; to |x| = 1 the same
 *          reduction with the exact (2^q 2^(j/64) - 1) first, so small
 *          results keep their relative precision; beyond, exp - 1.
 *   log    x = 2^e m, F = 1 + j/128 the table point nearest m (halved with
 *          m for m >= 1.5), ln x = e ln2 + ln F + ln(1 + r), r = (m - F)/F
 *          (m - F exact, |r| <= 1/192), ln F a double-double from the
 *          table, ln(1 + r) to degree 8.
 *   lfact  log(k!) exactly from the double k! for k < 20, else Stirling's
 *          series for log Gamma(k+1) to the x^-7 term.
 * Every polynomial is evaluated by Estrin's scheme.
 * Accuracy is a few ulp; the tests compare against numpy.
 */
#ifndef LPG_DETMATH_H
#define LPG_DETMATH_H

#include <stdint.h>

#if defined(__CUDACC__)
#define LPG_HD __host__ __device__ __forceinline__
#else
#define LPG_HD static inline
#endif

#if !defined(__CUDACC__)
#include <math.h>
#include <string.h>
#endif

/* ln 2 split: LN2_HI = ln2 rounded to double with its low 20 mantissa bits
 * cleared; LN2_LO = ln2 - LN2_HI rounded to double. */
#define LPG_LN2_HI 0x1.62e42fef00000p-1
#define LPG_LN2_LO 0x1.473de6af278edp-34
#define LPG_INV_LN2 0x1.71547652b82fep+0
#define LPG_SQRT2 0x1.6a09e667f3bcdp+0
#define LPG_HALF_LOG_2PI 0x1.d67f1c864beb5p-1

LPG_HD uint64_t lpg_dbits(double x) {
#if defined(__CUDA_ARCH__)
  return (uint64_t)__double_as_longlong(x);
#else
  uint64_t u;
  memcpy(&u, &x, sizeof u);
  return u;
#endif
}

LPG_HD double lpg_bitsd(uint64_t u) {
#if defined(__CUDA_ARCH__)
  return __longlong_as_double((long long)u);
#else
  double x;
  memcpy(&x, &u, sizeof x);
  return x;
#endif
}

/* 2^k for -1022 <= k <= 1023, built from the exponent field. */
LPG_HD double lpg_pow2i(int k) { return lpg_bitsd((uint64_t)(k + 1023) << 52); }

/* p * 2^k, exact whenever the result is a normal double. */
LPG_HD double lpg_scale2(double p, int k) {
  if (k > 1023) return (p * lpg_pow2i(1023)) * lpg_pow2i(k - 1023);
  if (k < -1022) return (p * lpg_pow2i(k + 600)) * lpg_pow2i(-600);
  return p * lpg_pow2i(k);
}

/* Tables (gen_detmath_tables.py, correctly rounded from 60-digit decimal
 * arithmetic): ln F_j as double-doubles and 1/F_j for the 129 log points,
 * F_j = 1 + j/128 (j < 64) or (1 + j/128)/2 (j >= 64); 2^(j/64) as
 * double-doubles for exp; ln k! for k < 256. */
#define LPG_INIT_LOG_HI \
  { \
  0x0.0p+0, 0x1.fe02a6b106789p-8, 0x1.fc0a8b0fc03e4p-7, 0x1.7b91b07d5b11bp-6, \
  0x1.f829b0e783300p-6, 0x1.39e87b9febd60p-5, 0x1.77458f632dcfcp-5, 0x1.b42dd711971bfp-5, \
  0x1.f0a30c01162a6p-5, 0x1.16536eea37ae1p-4, 0x1.341d7961bd1d1p-4, 0x1.51b073f06183fp-4, \
  0x1.6f0d28ae56b4cp-4, 0x1.8c345d6319b21p-4, 0x1.a926d3a4ad563p-4, 0x1.c5e548f5bc743p-4, \
  0x1.e27076e2af2e6p-4, 0x1.fec9131dbeabbp-4, 0x1.0d77e7cd08e59p-3, 0x1.1b72ad52f67a0p-3, \
  0x1.29552f81ff523p-3, 0x1.371fc201e8f74p-3, 0x1.44d2b6ccb7d1ep-3, 0x1.526e5e3a1b438p-3, \
  0x1.5ff3070a793d4p-3, 0x1.6d60fe719d21dp-3, 0x1.7ab890210d909p-3, 0x1.87fa06520c911p-3, \
  0x1.9525a9cf456b4p-3, 0x1.a23bc1fe2b563p-3, 0x1.af3c94e80bff3p-3, 0x1.bc286742d8cd6p-3, \
  0x1.c8ff7c79a9a22p-3, 0x1.d5c216b4fbb91p-3, 0x1.e27076e2af2e6p-3, 0x1.ef0adcbdc5936p-3, \
  0x1.fb9186d5e3e2bp-3, 0x1.0402594b4d041p-2, 0x1.0a324e27390e3p-2, 0x1.1058bf9ae4ad5p-2, \
  0x1.1675cababa60ep-2, 0x1.1c898c16999fbp-2, 0x1.22941fbcf7966p-2, 0x1.2895a13de86a3p-2, \
  0x1.2e8e2bae11d31p-2, 0x1.347dd9a987d55p-2, 0x1.3a64c556945eap-2, 0x1.404308686a7e4p-2, \
  0x1.4618bc21c5ec2p-2, 0x1.4be5f957778a1p-2, 0x1.51aad872df82dp-2, 0x1.5767717455a6cp-2, \
  0x1.5d1bdbf5809cap-2, 0x1.62c82f2b9c795p-2, 0x1.686c81e9b14afp-2, 0x1.6e08eaa2ba1e4p-2, \
  0x1.739d7f6bbd007p-2, 0x1.792a55fdd47a2p-2, 0x1.7eaf83b82afc3p-2, 0x1.842d1da1e8b17p-2, \
  0x1.89a3386c1425bp-2, 0x1.8f11e873662c7p-2, 0x1.947941c2116fbp-2, 0x1.99d958117e08bp-2, \
  -0x1.269621134db92p-2, -0x1.214456d0eb8d4p-2, -0x1.1bf99635a6b95p-2, -0x1.16b5ccbacfb73p-2, \
  -0x1.1178e8227e47cp-2, -0x1.0c42d676162e3p-2, -0x1.07138604d5862p-2, -0x1.01eae5626c691p-2, \
  -0x1.f991c6cb3b379p-3, -0x1.ef5ade4dcffe6p-3, -0x1.e530effe71012p-3, -0x1.db13db0d48940p-3, \
  -0x1.d1037f2655e7bp-3, -0x1.c6ffbc6f00f71p-3, -0x1.bd087383bd8adp-3, -0x1.b31d8575bce3dp-3, \
  -0x1.a93ed3c8ad9e3p-3, -0x1.9f6c407089664p-3, -0x1.95a5adcf7017fp-3, -0x1.8beafeb38fe8cp-3, \
  -0x1.823c16551a3c2p-3, -0x1.7898d85444c73p-3, -0x1.6f0128b756abcp-3, -0x1.6574ebe8c133ap-3, \
  -0x1.5bf406b543db2p-3, -0x1.527e5e4a1b58dp-3, -0x1.4913d8333b561p-3, -0x1.3fb45a59928ccp-3, \
  -0x1.365fcb0159016p-3, -0x1.2d1610c86813ap-3, -0x1.23d712a49c202p-3, -0x1.1aa2b7e23f72ap-3, \
  -0x1.1178e8227e47cp-3, -0x1.08598b59e3a07p-3, -0x1.fe89139dbd566p-4, -0x1.ec739830a1120p-4, \
  -0x1.da727638446a2p-4, -0x1.c885801bc4b23p-4, -0x1.b6ac88dad5b1cp-4, -0x1.a4e7640b1bc38p-4, \
  -0x1.9335e5d594989p-4, -0x1.8197e2f40e3f0p-4, -0x1.700d30aeac0e1p-4, -0x1.5e95a4d9791cbp-4, \
  -0x1.4d3115d207eacp-4, -0x1.3bdf5a7d1ee64p-4, -0x1.2aa04a44717a5p-4, -0x1.1973bd1465567p-4, \
  -0x1.08598b59e3a07p-4, -0x1.eea31c006b87cp-5, -0x1.ccb73cdddb2ccp-5, -0x1.aaef2d0fb10fcp-5, \
  -0x1.894aa149fb343p-5, -0x1.67c94f2d4bb58p-5, -0x1.466aed42de3eap-5, -0x1.252f32f8d183fp-5, \
  -0x1.0415d89e74444p-5, -0x1.c63d2ec14aaf2p-6, -0x1.8492528c8cabfp-6, -0x1.432a925980cc1p-6, \
  -0x1.0205658935847p-6, -0x1.82448a388a2aap-7, -0x1.010157588de71p-7, -0x1.0080559588b35p-8, \
  0x0.0p+0 \
  }

#define LPG_INIT_LOG_LO \
  { \
  0x0.0p+0, -0x1.e44b7e3711ebfp-67, -0x1.83092c59642a1p-62, -0x1.5b602ace3a510p-60, \
  0x1.33e3f04f1ef23p-60, -0x1.5bfa937f551bbp-59, 0x1.18d3ca87b9296p-59, -0x1.eb9759c130499p-60, \
  0x1.85f325c5bbacdp-59, -0x1.79da3e8c22cdap-60, -0x1.b599f227becbbp-58, 0x1.a49e39a1a8be4p-58, \
  -0x1.906d99184b992p-58, -0x1.4a697ab3424a9p-61, 0x1.942f48aa70ea9p-58, 0x1.5d617ef8161b1p-60, \
  -0x1.61578001e0162p-60, -0x1.5746b9981b36cp-58, 0x1.9a5dc5e9030acp-57, 0x1.483023472cd74p-58, \
  0x1.301771c407dbfp-57, 0x1.de6cb62af18a0p-58, 0x1.9f4f6543e1f88p-57, -0x1.746ff8a470d3ap-57, \
  -0x1.bc60efafc6f6ep-58, -0x1.caae268ecd179p-57, 0x1.be36b2d6a0608p-59, -0x1.bf7fdbfa08d9ap-57, \
  0x1.d904c1d4e2e26p-57, 0x1.93711b07a998cp-59, -0x1.398cff3641985p-58, 0x1.4fce744870f55p-58, \
  -0x1.4f689f8434012p-57, 0x1.6e443597e4d40p-57, -0x1.61578001e0162p-59, 0x1.48637950dc20dp-57, \
  -0x1.caaae64f21acbp-57, -0x1.28ec217a5022dp-57, 0x1.7dcfde8061c03p-56, 0x1.89fa0ab4cb31dp-58, \
  0x1.ce63eab883717p-61, -0x1.0e5c62aff1c44p-60, -0x1.76f5eb09628afp-56, 0x1.7ad24c13f040ep-56, \
  -0x1.8f4cdb95ebdf9p-56, -0x1.4dd4c580919f8p-57, -0x1.c68651945f97cp-57, -0x1.0bcfb6082ce6dp-56, \
  0x1.f42decdeccf1dp-56, -0x1.259b35b04813dp-57, 0x1.3927ac19f55e3p-59, 0x1.526adb283660cp-56, \
  0x1.4236383dc7fe1p-56, 0x1.7b7af915300e5p-57, -0x1.ddea0f7f58e3dp-57, -0x1.cfb1b39ca3a0fp-56, \
  -0x1.8c76ceb014b04p-56, 0x1.f057691fe9ed7p-56, 0x1.92ce979ed2950p-56, 0x1.24ec519784676p-56, \
  -0x1.29639dfbbf0fbp-56, 0x1.f85da755a61a3p-56, -0x1.16cc8bae0bbe4p-56, -0x1.a2b6889dc3e72p-57, \
  -0x1.e0efadd9db02bp-56, -0x1.f7ae91aeba60ap-57, 0x1.12aeb84249223p-57, -0x1.66fbd28b40935p-56, \
  0x1.0e63a5f01c691p-57, -0x1.162c79d5d11eep-58, -0x1.cdb16ed4e9138p-56, 0x1.18290bd2932e2p-59, \
  -0x1.f665066f980a2p-57, 0x1.08ab2ddc708a0p-58, -0x1.2276041f43042p-59, -0x1.aa11d49f96cb9p-58, \
  -0x1.60629242471a2p-57, 0x1.8e58b2c57a4a5p-57, -0x1.dd355f6a516d7p-60, 0x1.6353ab386a94dp-57, \
  -0x1.bcafa9de97203p-57, -0x1.35a19605e67efp-59, -0x1.142c507fb7a3dp-58, -0x1.55aa8b6997a40p-58, \
  0x1.1232ce70be781p-57, -0x1.ef8f6ebcfb201p-58, 0x1.8de59c21e166cp-57, 0x1.d34f0f4621bedp-60, \
  0x1.1f5b44c0df7e7p-61, 0x1.71a9682395bfdp-61, 0x1.0d5604930f135p-58, 0x1.d87e6a354d056p-57, \
  -0x1.7d411a5b944adp-58, 0x1.499a3f25af95fp-58, 0x1.6e38161051d69p-57, 0x1.c6ef1d9b2ef7ep-59, \
  0x1.0e63a5f01c691p-58, 0x1.dd7009902bf32p-57, 0x1.ac9f4215f9393p-58, 0x1.a2bf991780d3fp-59, \
  -0x1.401fa71733019p-58, -0x1.a38cb559a6706p-58, 0x1.0057eed1ca59fp-59, 0x1.5b5ca203e4259p-58, \
  0x1.478a85704ccb7p-58, -0x1.b9f2dffbeed43p-60, 0x1.72566212cdd05p-61, -0x1.f38745c5c450ap-58, \
  -0x1.769f42c7842ccp-58, -0x1.7a976d3b5b45fp-59, 0x1.d15d38d2fa3f7p-58, 0x1.7558367a6acf6p-59, \
  0x1.dd7009902bf32p-58, 0x1.3e4fc93b7b66cp-59, 0x1.e48fb0500efd4p-59, -0x1.a353bb42e0addp-61, \
  -0x1.a8be97660a23dp-60, -0x1.0413e6505e603p-59, 0x1.cdd6f7f4a137ep-59, 0x1.947f792615916p-59, \
  -0x1.c05cf1d753622p-59, 0x1.ce030a686bd86p-60, 0x1.d192d0619fa67p-60, 0x1.8cdaf39004192p-60, \
  -0x1.27c8e8416e71fp-60, -0x1.04b16137f09a0p-62, -0x1.46662d417ced0p-62, -0x1.f96638cf63677p-62, \
  0x0.0p+0 \
  }

#define LPG_INIT_INV \
  { \
  0x1.0000000000000p+0, 0x1.fc07f01fc07f0p-1, 0x1.f81f81f81f820p-1, 0x1.f44659e4a4271p-1, \
  0x1.f07c1f07c1f08p-1, 0x1.ecc07b301ecc0p-1, 0x1.e9131abf0b767p-1, 0x1.e573ac901e574p-1, \
  0x1.e1e1e1e1e1e1ep-1, 0x1.de5d6e3f8868ap-1, 0x1.dae6076b981dbp-1, 0x1.d77b654b82c34p-1, \
  0x1.d41d41d41d41dp-1, 0x1.d0cb58f6ec074p-1, 0x1.cd85689039b0bp-1, 0x1.ca4b3055ee191p-1, \
  0x1.c71c71c71c71cp-1, 0x1.c3f8f01c3f8f0p-1, 0x1.c0e070381c0e0p-1, 0x1.bdd2b899406f7p-1, \
  0x1.bacf914c1bad0p-1, 0x1.b7d6c3dda338bp-1, 0x1.b4e81b4e81b4fp-1, 0x1.b2036406c80d9p-1, \
  0x1.af286bca1af28p-1, 0x1.ac5701ac5701bp-1, 0x1.a98ef606a63bep-1, 0x1.a6d01a6d01a6dp-1, \
  0x1.a41a41a41a41ap-1, 0x1.a16d3f97a4b02p-1, 0x1.9ec8e951033d9p-1, 0x1.9c2d14ee4a102p-1, \
  0x1.999999999999ap-1, 0x1.970e4f80cb872p-1, 0x1.948b0fcd6e9e0p-1, 0x1.920fb49d0e229p-1, \
  0x1.8f9c18f9c18fap-1, 0x1.8d3018d3018d3p-1, 0x1.8acb90f6bf3aap-1, 0x1.886e5f0abb04ap-1, \
  0x1.8618618618618p-1, 0x1.83c977ab2beddp-1, 0x1.8181818181818p-1, 0x1.7f405fd017f40p-1, \
  0x1.7d05f417d05f4p-1, 0x1.7ad2208e0ecc3p-1, 0x1.78a4c8178a4c8p-1, 0x1.767dce434a9b1p-1, \
  0x1.745d1745d1746p-1, 0x1.724287f46debcp-1, 0x1.702e05c0b8170p-1, 0x1.6e1f76b4337c7p-1, \
  0x1.6c16c16c16c17p-1, 0x1.6a13cd1537290p-1, 0x1.6816816816817p-1, 0x1.661ec6a5122f9p-1, \
  0x1.642c8590b2164p-1, 0x1.623fa77016240p-1, 0x1.6058160581606p-1, 0x1.5e75bb8d015e7p-1, \
  0x1.5c9882b931057p-1, 0x1.5ac056b015ac0p-1, 0x1.58ed2308158edp-1, 0x1.571ed3c506b3ap-1, \
  0x1.5555555555555p+0, 0x1.5390948f40febp+0, 0x1.51d07eae2f815p+0, 0x1.5015015015015p+0, \
  0x1.4e5e0a72f0539p+0, 0x1.4cab88725af6ep+0, 0x1.4afd6a052bf5bp+0, 0x1.49539e3b2d067p+0, \
  0x1.47ae147ae147bp+0, 0x1.460cbc7f5cf9ap+0, 0x1.446f86562d9fbp+0, 0x1.42d6625d51f87p+0, \
  0x1.4141414141414p+0, 0x1.3fb013fb013fbp+0, 0x1.3e22cbce4a902p+0, 0x1.3c995a47babe7p+0, \
  0x1.3b13b13b13b14p+0, 0x1.3991c2c187f63p+0, 0x1.3813813813814p+0, 0x1.3698df3de0748p+0, \
  0x1.3521cfb2b78c1p+0, 0x1.33ae45b57bcb2p+0, 0x1.323e34a2b10bfp+0, 0x1.30d190130d190p+0, \
  0x1.2f684bda12f68p+0, 0x1.2e025c04b8097p+0, 0x1.2c9fb4d812ca0p+0, 0x1.2b404ad012b40p+0, \
  0x1.29e4129e4129ep+0, 0x1.288b01288b013p+0, 0x1.27350b8812735p+0, 0x1.25e22708092f1p+0, \
  0x1.2492492492492p+0, 0x1.23456789abcdfp+0, 0x1.21fb78121fb78p+0, 0x1.20b470c67c0d9p+0, \
  0x1.1f7047dc11f70p+0, 0x1.1e2ef3b3fb874p+0, 0x1.1cf06ada2811dp+0, 0x1.1bb4a4046ed29p+0, \
  0x1.1a7b9611a7b96p+0, 0x1.19453808ca29cp+0, 0x1.1811811811812p+0, 0x1.16e0689427379p+0, \
  0x1.15b1e5f75270dp+0, 0x1.1485f0e0acd3bp+0, 0x1.135c81135c811p+0, 0x1.12358e75d3033p+0, \
  0x1.1111111111111p+0, 0x1.0fef010fef011p+0, 0x1.0ecf56be69c90p+0, 0x1.0db20a88f4696p+0, \
  0x1.0c9714fbcda3bp+0, 0x1.0b7e6ec259dc8p+0, 0x1.0a6810a6810a7p+0, 0x1.0953f39010954p+0, \
  0x1.0842108421084p+0, 0x1.073260a47f7c6p+0, 0x1.0624dd2f1a9fcp+0, 0x1.05197f7d73404p+0, \
  0x1.0410410410410p+0, 0x1.03091b51f5e1ap+0, 0x1.0204081020408p+0, 0x1.0101010101010p+0, \
  0x1.0000000000000p+0 \
  }

#define LPG_INIT_EXP_HI \
  { \
  0x1.0000000000000p+0, 0x1.02c9a3e778061p+0, 0x1.059b0d3158574p+0, 0x1.0874518759bc8p+0, \
  0x1.0b5586cf9890fp+0, 0x1.0e3ec32d3d1a2p+0, 0x1.11301d0125b51p+0, 0x1.1429aaea92de0p+0, \
  0x1.172b83c7d517bp+0, 0x1.1a35beb6fcb75p+0, 0x1.1d4873168b9aap+0, 0x1.2063b88628cd6p+0, \
  0x1.2387a6e756238p+0, 0x1.26b4565e27cddp+0, 0x1.29e9df51fdee1p+0, 0x1.2d285a6e4030bp+0, \
  0x1.306fe0a31b715p+0, 0x1.33c08b26416ffp+0, 0x1.371a7373aa9cbp+0, 0x1.3a7db34e59ff7p+0, \
  0x1.3dea64c123422p+0, 0x1.4160a21f72e2ap+0, 0x1.44e086061892dp+0, 0x1.486a2b5c13cd0p+0, \
  0x1.4bfdad5362a27p+0, 0x1.4f9b2769d2ca7p+0, 0x1.5342b569d4f82p+0, 0x1.56f4736b527dap+0, \
  0x1.5ab07dd485429p+0, 0x1.5e76f15ad2148p+0, 0x1.6247eb03a5585p+0, 0x1.6623882552225p+0, \
  0x1.6a09e667f3bcdp+0, 0x1.6dfb23c651a2fp+0, 0x1.71f75e8ec5f74p+0, 0x1.75feb564267c9p+0, \
  0x1.7a11473eb0187p+0, 0x1.7e2f336cf4e62p+0, 0x1.82589994cce13p+0, 0x1.868d99b4492edp+0, \
  0x1.8ace5422aa0dbp+0, 0x1.8f1ae99157736p+0, 0x1.93737b0cdc5e5p+0, 0x1.97d829fde4e50p+0, \
  0x1.9c49182a3f090p+0, 0x1.a0c667b5de565p+0, 0x1.a5503b23e255dp+0, 0x1.a9e6b5579fdbfp+0, \
  0x1.ae89f995ad3adp+0, 0x1.b33a2b84f15fbp+0, 0x1.b7f76f2fb5e47p+0, 0x1.bcc1e904bc1d2p+0, \
  0x1.c199bdd85529cp+0, 0x1.c67f12e57d14bp+0, 0x1.cb720dcef9069p+0, 0x1.d072d4a07897cp+0, \
  0x1.d5818dcfba487p+0, 0x1.da9e603db3285p+0, 0x1.dfc97337b9b5fp+0, 0x1.e502ee78b3ff6p+0, \
  0x1.ea4afa2a490dap+0, 0x1.efa1bee615a27p+0, 0x1.f50765b6e4540p+0, 0x1.fa7c1819e90d8p+0 \
  }

#define LPG_INIT_EXP_LO \
  { \
  0x0.0p+0, -0x1.19083535b085dp-56, 0x1.d73e2a475b465p-55, 0x1.186be4bb284ffp-57, \
  0x1.8a62e4adc610bp-54, 0x1.03a1727c57b53p-59, -0x1.6c51039449b3ap-54, -0x1.32fbf9af1369ep-54, \
  -0x1.19041b9d78a76p-55, 0x1.e5b4c7b4968e4p-55, 0x1.e016e00a2643cp-54, 0x1.dc775814a8495p-55, \
  0x1.9b07eb6c70573p-54, 0x1.2bd339940e9d9p-55, 0x1.612e8afad1255p-55, 0x1.0024754db41d5p-54, \
  0x1.6f46ad23182e4p-55, 0x1.32721843659a6p-54, -0x1.63aeabf42eae2p-54, -0x1.5e436d661f5e3p-56, \
  0x1.ada0911f09ebcp-55, -0x1.ef3691c309278p-58, 0x1.89b7a04ef80d0p-59, 0x1.3c1a3b69062f0p-56, \
  0x1.d4397afec42e2p-56, -0x1.4b309d25957e3p-54, -0x1.07abe1db13cadp-55, 0x1.9bb2c011d93adp-54, \
  0x1.6324c054647adp-54, 0x1.ba6f93080e65ep-54, -0x1.383c17e40b497p-54, -0x1.bb60987591c34p-54, \
  -0x1.bdd3413b26456p-54, -0x1.bbe3a683c88abp-57, -0x1.16e4786887a99p-55, -0x1.0245957316dd3p-54, \
  -0x1.41577ee04992fp-55, 0x1.05d02ba15797ep-56, -0x1.d4c1dd41532d8p-54, -0x1.fc6f89bd4f6bap-54, \
  0x1.6e9f156864b27p-54, 0x1.5cc13a2e3976cp-55, -0x1.75fc781b57ebcp-57, -0x1.d185b7c1b85d1p-54, \
  0x1.c7c46b071f2bep-56, -0x1.359495d1cd533p-54, -0x1.d2f6edb8d41e1p-54, 0x1.0fac90ef7fd31p-54, \
  0x1.7a1cd345dcc81p-54, -0x1.2805e3084d708p-57, -0x1.5584f7e54ac3bp-56, 0x1.23dd07a2d9e84p-55, \
  0x1.11065895048ddp-55, 0x1.2884dff483cadp-54, 0x1.503cbd1e949dbp-56, -0x1.cbc3743797a9cp-54, \
  0x1.2ed02d75b3707p-55, 0x1.c2300696db532p-54, -0x1.1a5cd4f184b5cp-54, 0x1.39e8980a9cc8fp-55, \
  -0x1.e9c23179c2893p-54, 0x1.dc7f486a4b6b0p-54, 0x1.9d3e12dd8a18bp-54, 0x1.74853f3a5931ep-55 \
  }

#define LPG_INIT_LFACT \
  { \
  0x0.0p+0, 0x0.0p+0, 0x1.62e42fefa39efp-1, 0x1.cab0bfa2a2002p+0, \
  0x1.96ca77c922cf9p+1, 0x1.326643c4479c9p+2, 0x1.a51273acf01cap+2, 0x1.10ce1f32dcc30p+3, \
  0x1.5358e82fcb70dp+3, 0x1.99a8921a7f7cfp+3, 0x1.e357590954d15p+3, 0x1.180973f3a8d74p+4, \
  0x1.3fcba16d50143p+4, 0x1.68d5a9c3b32cep+4, 0x1.930f3df162a42p+4, 0x1.be636a63fd346p+4, \
  0x1.eabff061f1a84p+4, 0x1.0c0a63f2f353ap+5, 0x1.2329df2d5ee52p+5, 0x1.3ab8153363985p+5, \
  0x1.52af57aed77bep+5, 0x1.6b0a8643472a9p+5, 0x1.83c4faba84f06p+5, 0x1.9cda78b856a45p+5, \
  0x1.b6472034e8d14p+5, 0x1.d007622cd65e7p+5, 0x1.ea17f717c6794p+5, 0x1.023aeb67e4fefp+6, \
  0x1.0f8f18d330240p+6, 0x1.1d07353917231p+6, 0x1.2aa208b59d0e5p+6, 0x1.385e6fd9e5a40p+6, \
  0x1.463b59b942084p+6, 0x1.5437c633ace4ap+6, 0x1.6252c474896bap+6, 0x1.708b719e11658p+6, \
  0x1.7ee0f79b26758p+6, 0x1.8d528c1243d96p+6, 0x1.9bdf6f75257a3p+6, 0x1.aa86ec2969812p+6, \
  0x1.b94855c702ba2p+6, 0x1.c8230869ca105p+6, 0x1.d7166813e12eep+6, 0x1.e621e01eeba4fp+6, \
  0x1.f544e2ba69cf1p+6, 0x1.023f743addd9fp+7, 0x1.09e7b7ea41ea9p+7, 0x1.119afe762626bp+7, \
  0x1.19590c853a559p+7, 0x1.2121a930c6ec3p+7, 0x1.28f49ddeb1f31p+7, 0x1.30d1b61e86335p+7, \
  0x1.38b8bf8931ddbp+7, 0x1.40a989a33a6cdp+7, 0x1.48a3e5c12af19p+7, 0x1.50a7a6ee08711p+7, \
  0x1.58b4a1d39da73p+7, 0x1.60caaca474746p+7, 0x1.68e99f0757979p+7, 0x1.711152043b2c4p+7, \
  0x1.79419ff26dc59p+7, 0x1.817a6467f6fb9p+7, 0x1.89bb7c2a0aea1p+7, 0x1.9204c51e7c761p+7, \
  0x1.9a561e3e1a4bdp+7, 0x1.a2af6787e4609p+7, 0x1.ab1081f509726p+7, 0x1.b3794f6d9d7afp+7, \
  0x1.bbe9b2bdfb621p+7, 0x1.c4618f8cc56f7p+7, 0x1.cce0ca5179100p+7, 0x1.d567484b8b7b6p+7, \
  0x1.ddf4ef7a05a70p+7, 0x1.e689a69396befp+7, 0x1.ef2554ff15148p+7, 0x1.f7c7e2cc66183p+7, \
  0x1.00389c56e3462p+8, 0x1.04909ff8b652bp+8, 0x1.08ebf13dbf263p+8, 0x1.0d4a85602b129p+8, \
  0x1.11ac51df8932ap+8, 0x1.16114c7e34736p+8, 0x1.1a796b3ede1acp+8, 0x1.1ee4a46236d3ep+8, \
  0x1.2352ee64b46d5p+8, 0x1.27c43ffc72962p+8, 0x1.2c3890172d057p+8, 0x1.30afd5d851956p+8, \
  0x1.352a089728f1bp+8, 0x1.39a71fdd14947p+8, 0x1.3e271363e0df7p+8, 0x1.42a9db142a36ap+8, \
  0x1.472f6f03d410cp+8, 0x1.4bb7c77491066p+8, 0x1.5042dcd27af64p+8, 0x1.54d0a7b2ba658p+8, \
  0x1.596120d23c4ecp+8, 0x1.5df4411475a1cp+8, 0x1.628a018233bedp+8, 0x1.67225b4879462p+8, \
  0x1.6bbd47b7669b6p+8, 0x1.705ac0412d89fp+8, 0x1.74fabe790f7bep+8, 0x1.799d3c1265c0ep+8, \
  0x1.7e4232dfb367dp+8, 0x1.82e99cd1c0368p+8, 0x1.879373f6bc4fep+8, 0x1.8c3fb2796c21cp+8, \
  0x1.90ee52a05c35fp+8, 0x1.959f4ecd1c8b3p+8, 0x1.9a52a17b831ccp+8, 0x1.9f084540f545ep+8, \
  0x1.a3c034cbb7b2cp+8, 0x1.a87a6ae24493ap+8, 0x1.ad36e262a7cc0p+8, 0x1.b1f59641e0db5p+8, \
  0x1.b6b6818b4a3ebp+8, 0x1.bb799f600610ap+8, 0x1.c03eeaf66facdp+8, 0x1.c5065f9992226p+8, \
  0x1.c9cff8a8a340dp+8, 0x1.ce9bb196830eap+8, 0x1.d36985e93f7b8p+8, 0x1.d83971399c213p+8, \
  0x1.dd0b6f329dea4p+8, 0x1.e1df7b911a74cp+8, 0x1.e6b592234b0c9p+8, 0x1.eb8daec863182p+8, \
  0x1.f067cd7029d4dp+8, 0x1.f543ea1a97428p+8, 0x1.fa2200d7741ebp+8, 0x1.ff020dc5fcd0cp+8, \
  0x1.01f2068a4395cp+9, 0x1.0463fd801573cp+9, 0x1.06d6e9ea365edp+9, 0x1.094ac9f576038p+9, \
  0x1.0bbf9bd589663p+9, 0x1.0e355dc4e4164p+9, 0x1.10ac0e0492828p+9, 0x1.1323aadc1563ep+9, \
  0x1.159c32993e34fp+9, 0x1.1815a3900cac1p+9, 0x1.1a8ffc1a8d2fep+9, 0x1.1d0b3a98b83c1p+9, \
  0x1.1f875d7052afep+9, 0x1.2204630ccefc3p+9, 0x1.248249df2f2b1p+9, 0x1.2701105de7b8dp+9, \
  0x1.2980b504c3372p+9, 0x1.2c013654c6b40p+9, 0x1.2e8292d416dddp+9, 0x1.3104c90dddddep+9, \
  0x1.3387d79231e3dp+9, 0x1.360bbcf5fc5bfp+9, 0x1.389077d2e1cb2p+9, 0x1.3b1606c72a4a4p+9, \
  0x1.3d9c6875aa9cfp+9, 0x1.40239b85adddfp+9, 0x1.42ab9ea2dfbd1p+9, 0x1.4534707d3748fp+9, \
  0x1.47be0fc8e241ep+9, 0x1.4a487b3e30effp+9, 0x1.4cd3b19982794p+9, 0x1.4f5fb19b31b3fp+9, \
  0x1.51ec7a0782708p+9, 0x1.547a09a68f387p+9, 0x1.57085f44377dfp+9, 0x1.599779b00e38ep+9, \
  0x1.5c2757bd48ee8p+9, 0x1.5eb7f842af200p+9, 0x1.61495a1a8a1d5p+9, 0x1.63db7c229538bp+9, \
  0x1.666e5d3bee594p+9, 0x1.6901fc4b06e89p+9, 0x1.6b96583795197p+9, 0x1.6e2b6fec85852p+9, \
  0x1.70c14257ed1c3p+9, 0x1.7357ce6afb697p+9, 0x1.75ef1319ed23cp+9, 0x1.78870f5bff0cdp+9, \
  0x1.7b1fc22b611b3p+9, 0x1.7db92a8529ed1p+9, 0x1.805347694a819p+9, 0x1.82ee17da82373p+9, \
  0x1.85899ade530d2p+9, 0x1.8825cf7cf6261p+9, 0x1.8ac2b4c15089cp+9, 0x1.8d6049b8e8253p+9, \
  0x1.8ffe8d73d9061p+9, 0x1.929d7f04cad12p+9, 0x1.953d1d80e671bp+9, 0x1.97dd67ffcbffcp+9, \
  0x1.9a7e5d9b88dd4p+9, 0x1.9d1ffd708e071p+9, 0x1.9fc2469da6998p+9, 0x1.a2653843ee86cp+9, \
  0x1.a508d186c97e3p+9, 0x1.a7ad118bda02bp+9, 0x1.aa51f77af8af4p+9, 0x1.acf7827e2ba8fp+9, \
  0x1.af9db1c19e3c7p+9, 0x1.b244847398a6bp+9, 0x1.b4ebf9c47806ep+9, 0x1.b79410e6a6799p+9, \
  0x1.ba3cc90e935b7p+9, 0x1.bce62172abb2ap+9, 0x1.bf90194b52be1p+9, 0x1.c23aafd2daa98p+9, \
  0x1.c4e5e4457d65ep+9, 0x1.c791b5e155a48p+9, 0x1.ca3e23e657f4cp+9, 0x1.cceb2d964c030p+9, \
  0x1.cf98d234c5f8ap+9, 0x1.d24711071ffb9p+9, 0x1.d4f5e95473cd6p+9, 0x1.d7a55a6594889p+9, \
  0x1.da556385087b9p+9, 0x1.dd0603ff03211p+9, 0x1.dfb73b215f34ap+9, 0x1.e269083b98e2bp+9, \
  0x1.e51b6a9ec8146p+9, 0x1.e7ce619d9ad52p+9, 0x1.ea81ec8c4fd29p+9, 0x1.ed360ac0b0f5ep+9, \
  0x1.efeabb920e153p+9, 0x1.f29ffe5937be4p+9, 0x1.f555d2707a179p+9, 0x1.f80c373397d9cp+9, \
  0x1.fac32bffc55eep+9, 0x1.fd7ab033a3c7fp+9, 0x1.001961979e1c4p+10, 0x1.0175b229fd937p+10, \
  0x1.02d2498255e0cp+10, 0x1.042f2752b9b42p+10, 0x1.058c4b4de69d1p+10, 0x1.06e9b52742dadp+10, \
  0x1.08476492db365p+10, 0x1.09a5594560e57p+10, 0x1.0b0392f427775p+10, 0x1.0c62115522c95p+10, \
  0x1.0dc0d41ee5056p+10, 0x1.0f1fdb089ca83p+10, 0x1.107f25ca12901p+10, 0x1.11deb41ba8145p+10, \
  0x1.133e85b655240p+10, 0x1.149e9a53a66d0p+10, 0x1.15fef1adbb8aep+10, 0x1.175f8b7f453cep+10, \
  0x1.18c0678383a39p+10, 0x1.1a2185764485fp+10, 0x1.1b82e513e19d0p+10, 0x1.1ce486193ee72p+10, \
  0x1.1e466843c9018p+10, 0x1.1fa88b517388ep+10, 0x1.210aef00b7803p+10, 0x1.226d931091be7p+10 \
  }

#if defined(__CUDACC__)
__constant__ double lpg_tab_lfact_dev[256] = LPG_INIT_LFACT;
__constant__ double lpg_tab_log_hi_dev[129] = LPG_INIT_LOG_HI;
__constant__ double lpg_tab_log_lo_dev[129] = LPG_INIT_LOG_LO;
__constant__ double lpg_tab_inv_dev[129] = LPG_INIT_INV;
__constant__ double lpg_tab_exp_hi_dev[64] = LPG_INIT_EXP_HI;
__constant__ double lpg_tab_exp_lo_dev[64] = LPG_INIT_EXP_LO;
#endif
static const double lpg_tab_lfact_host[256] = LPG_INIT_LFACT;
static const double lpg_tab_log_hi_host[129] = LPG_INIT_LOG_HI;
static const double lpg_tab_log_lo_host[129] = LPG_INIT_LOG_LO;
static const double lpg_tab_inv_host[129] = LPG_INIT_INV;
static const double lpg_tab_exp_hi_host[64] = LPG_INIT_EXP_HI;
static const double lpg_tab_exp_lo_host[64] = LPG_INIT_EXP_LO;
#if defined(__CUDA_ARCH__)
#define LPG_TAB(name) lpg_tab_##name##_dev
#else
#define LPG_TAB(name) lpg_tab_##name##_host
#endif

/* Polynomials by Estrin's scheme (pairs, then powers r^2, r^4): the same
 * polynomial as Horner's rule with a shorter dependency chain, which
 * matters on a GPU whose double-precision operations have a long latency.
 * The series are arranged as r + r^2 P(r) so that the dominant term r is
 * exact and the rounding of P is scaled down by r. */

/* e^r - 1 = r + r^2 (1/2 + r/6 + r^2/24 + r^3/120 + r^4/720) for
 * |r| <= ln2/128 (the omitted r^7/5040 is below 2^-60 of the result). */
LPG_HD double lpg_em1_small(double r) {
  const double r2 = r * r;
  const double q0 = 0.5 + (1.0 / 6.0) * r;
  const double q1 = (1.0 / 24.0) + (1.0 / 120.0) * r;
  const double s0 = q0 + q1 * r2;
  const double p = s0 + (1.0 / 720.0) * (r2 * r2);
  return r + r2 * p;
}

/* kd = round(x * 64 / ln2) split as kd = 64 q + j (0 <= j < 64), and the
 * reduced argument r = x - kd ln2/64 with a two-part ln2/64 (kd * hi exact
 * for |kd| < 2^20); |r| <= ln2/128 up to rounding. */
LPG_HD double lpg_exp_reduce(double x, int* q, int* j) {
  const double kd = floor(x * (64.0 * LPG_INV_LN2) + 0.5);
  const double r = (x - kd * (LPG_LN2_HI * 0x1.0p-6)) - kd * (LPG_LN2_LO * 0x1.0p-6);
  const int k = (int)kd;
  *j = k & 63;
  *q = (k - *j) / 64;
  return r;
}

/* e^x = 2^q 2^(j/64) e^r: table value times (1 + (e^r - 1)). */
LPG_HD double lpg_exp(double x) {
  if (x != x) return x;
  if (x > 709.782712893384) return lpg_bitsd(0x7ff0000000000000ULL);
  if (x < -745.2) return 0.0;
  int q, j;
  const double r = lpg_exp_reduce(x, &q, &j);
  const double p = lpg_em1_small(r);
  const double th = LPG_TAB(exp_hi)[j], tl = LPG_TAB(exp_lo)[j];
  return lpg_scale2(th + (tl + th * p), q);
}

/* e^x - 1: the short series for |x| <= ln2/128; up to |x| = 1 the reduced
 * form (2^q T - 1) + 2^q (T_lo + T p), whose first term is exact
 * (Sterbenz), so small results keep their relative precision; beyond, e^x - 1. */
LPG_HD double lpg_expm1(double x) {
  if (x != x) return x;
  if (x > -0x1.62e42fefa39efp-8 && x < 0x1.62e42fefa39efp-8) return lpg_em1_small(x);
  if (x < -40.0) return -1.0;
  if (x > 1.0 || x < -1.0) return lpg_exp(x) - 1.0;
  int q, j;
  const double r = lpg_exp_reduce(x, &q, &j);
  const double p = lpg_em1_small(r);
  const double s = lpg_pow2i(q);
  const double th = LPG_TAB(exp_hi)[j] * s, tl = LPG_TAB(exp_lo)[j] * s;
  return (th - 1.0) + (tl + th * p);
}

/* ln(1 + r) - r = r^2 (-1/2 + r/3 - r^2/4 + r^3/5 - r^4/6 + r^5/7 - r^6/8)
 * for |r| <= 1/192 (the omitted r^9/9 is below 2^-60 of r). */
LPG_HD double lpg_l1p_tail(double r) {
  const double r2 = r * r;
  const double r4 = r2 * r2;
  const double q0 = -0.5 + (1.0 / 3.0) * r;
  const double q1 = -0.25 + 0.2 * r;
  const double q2 = (-1.0 / 6.0) + (1.0 / 7.0) * r;
  const double s0 = q0 + q1 * r2;
  const double s1 = q2 + (-0.125) * r2;
  return r2 * (s0 + s1 * r4);
}

/* ln x = e ln2 + ln F_j + ln(1 + r), x = 2^e m, F_j = 1 + j/128 the table
 * point nearest m (for the upper half m and F_j halved and e raised, so
 * that a result near 0 never comes from cancelling e ln2 against ln F_j,
 * and x just below 1 meets F = 1 exactly), r = (m - F_j)/F_j with m - F_j
 * exact and |r| <= 1/192. */
LPG_HD double lpg_log(double x) {
  if (x != x) return x;
  if (x <= 0.0) return x == 0.0 ? -lpg_bitsd(0x7ff0000000000000ULL) : lpg_bitsd(0x7ff8000000000000ULL);
  if (x == lpg_bitsd(0x7ff0000000000000ULL)) return x;
  int eadj = 0;
  if (x < 0x1.0p-1022) { x = x * 0x1.0p54; eadj = -54; }
  const uint64_t b = lpg_dbits(x);
  int e = (int)((b >> 52) & 0x7ff) - 1023 + eadj;
  const uint64_t mant = b & 0x000fffffffffffffULL;
  const int j = (int)((mant + (1ULL << 44)) >> 45); /* 0 .. 128 */
  /* m in [1, 2) and F = 1 + j/128 from their bits, both halved (exponent
   * field 0x3fe) for j >= 64; F = 2/2 = 1 for j = 128 */
  const uint64_t ex = j >= 64 ? 0x3fe0000000000000ULL : 0x3ff0000000000000ULL;
  e += j >= 64 ? 1 : 0;
  const double m = lpg_bitsd(mant | ex);
  const double f = lpg_bitsd(ex + ((uint64_t)j << 45));
  const double r = (m - f) * LPG_TAB(inv)[j];
  const double ed = (double)e;
  const double hi = ed * LPG_LN2_HI + LPG_TAB(log_hi)[j];
  const double lo = (ed * LPG_LN2_LO + LPG_TAB(log_lo)[j]) + (r + lpg_l1p_tail(r));
  return hi + lo;
}

/* log(k!) for integer k >= 0. */
LPG_HD double lpg_lfact(int64_t k) {
  if (k < 2) return 0.0;
  if (k < 20) {
    double f = 1.0;
    for (int64_t i = 2; i <= k; ++i) f = f * (double)i; /* exact below 2^53 */
    return lpg_log(f);
  }
  double x = (double)(k + 1);
  double ix = 1.0 / x;
  double ix2 = ix * ix;
  double corr = ix * (1.0 / 12.0 - ix2 * (1.0 / 360.0 - ix2 * (1.0 / 1260.0 - ix2 * (1.0 / 1680.0))));
  return (x - 0.5) * lpg_log(x) - x + LPG_HALF_LOG_2PI + corr;
}

/* rint(r * 2^24) as an unsigned integer, clamped to [0, 2^62], for a float
 * r (0 for r <= 0 and NaN) — the fixed-point susceptibility weight — from
 * the bits of r alone, with integer operations only.  r * 2^24 is exact in
 * double, so this equals the double-precision definition
 * (d = (double)r * 2^24; !(d > 0) -> 0; min(d, 2^62); rint(d)) bit for bit:
 * for r = M * 2^(E - 150) (M the 24-bit significand, E the biased exponent)
 * the product is M * 2^(E - 126), a left shift for E >= 126 and otherwise a
 * right shift rounded half to even. */
LPG_HD uint64_t lpg_fix_risk_bits(float r) {
  union {
    float f;
    uint32_t u;
  } c;
  c.f = r;
  const uint32_t u = c.u;
  if (u & 0x80000000u) return 0; /* negative (or -0, negative NaN) */
  const uint32_t e = (u >> 23) & 0xffu;
  const uint32_t frac = u & 0x7fffffu;
  if (e == 0xffu) return frac ? 0 : ((uint64_t)1 << 62); /* NaN -> 0, +inf -> clamp */
  if (e == 0) return 0;                                   /* zero or subnormal: below 2^-126 * 2^24 < 1/2 */
  const uint64_t m = (uint64_t)(frac | 0x800000u);
  if (e >= 126) {
    const uint32_t sh = e - 126;
    if (sh >= 39) return (uint64_t)1 << 62; /* m * 2^sh >= 2^62 */
    const uint64_t v = m << sh;
    return v > ((uint64_t)1 << 62) ? ((uint64_t)1 << 62) : v;
  }
  const uint32_t s = 126 - e; /* 1 .. 125 */
  if (s > 24) return 0;       /* m * 2^-s < 1/2 */
  const uint64_t q = m >> s;
  const uint64_t rem = m & (((uint64_t)1 << s) - 1);
  const uint64_t half = (uint64_t)1 << (s - 1);
  return q + ((rem > half || (rem == half && (q & 1))) ? 1 : 0);
}

/* The same weight with single-precision arithmetic: r * 2^24 is exact in
 * float (a power-of-two scaling), and rounding an exact value to the nearest
 * integer, ties to even, gives the same integer in float as in double (below
 * 2^24 the result is representable; above 2^23 the value is already an
 * integer).  One multiply and one rounding conversion, no branches on the
 * bits. */
LPG_HD uint64_t lpg_fix_risk_f32(float r) {
  const float f = r * 16777216.0f;
  if (!(f > 0.0f)) return 0;
  if (f > 0x1.0p62f) return (uint64_t)1 << 62;
#if defined(__CUDA_ARCH__)
  /* the 32-bit conversion (single-precision path) whenever the integer fits:
   * every risk below 256; the 64-bit conversion is far slower on this GPU */
  if (f < 4294967296.0f) return (uint64_t)__float2uint_rn(f);
  return __float2ull_rn(f);
#else
  return (uint64_t)rintf(f);
#endif
}

/* ------------------------------------------------------------------------ */
/* Exact mixing of fixed-point infectivity over the network.
 *
 * A network weight w is held in two fixed-point parts, w = hi 2^-62 +
 * lo 2^-120: hi = floor(w 2^62) and lo the rest in units of 2^-120.  Both
 * steps are exact for every double w >= 2^-62 (scaling by a power of two is
 * exact, a double minus its floor is exact, and that fraction has at most 52
 * bits, so lo is an integer below 2^58); smaller weights are rounded to
 * 2^-120.  w >= 4 saturates hi (no row-normalised network reaches it).
 * A node's incoming infectivity sum_i B_i w_i (B in units of 2^-40) is then
 * A 2^-102 + R 2^-160 with A = sum_i B_i hi_i and R = sum_i B_i lo_i, each
 * summed exactly in three 64-bit words, so the result does not depend on
 * how the sum is split.  lpg_mix_value turns the two sums into one double
 * with a fixed sequence of roundings, identical on every target. */
LPG_HD void lpg_net_split(double w, uint64_t* hi, uint64_t* lo) {
  if (!(w > 0.0)) {
    *hi = 0;
    *lo = 0;
    return;
  }
  if (w >= 4.0) {
    *hi = 0xFFFFFFFFFFFFFFFFULL;
    *lo = 0;
    return;
  }
  const double s = w * 0x1.0p62;
  const double f = floor(s);
  *hi = (uint64_t)f;
  *lo = (uint64_t)rint((s - f) * 0x1.0p58);
}

/* (a2 2^128 + a1 2^64 + a0) 2^-102 + (r2 2^128 + r1 2^64 + r0) 2^-160 */
LPG_HD double lpg_mix_value(uint64_t a0, uint64_t a1, uint64_t a2, uint64_t r0, uint64_t r1, uint64_t r2) {
  const double A = ((double)a2 * 0x1.0p64 + (double)a1) * 0x1.0p64 + (double)a0;
  const double R = ((double)r2 * 0x1.0p64 + (double)r1) * 0x1.0p64 + (double)r0;
  return A * 0x1.0p-102 + R * 0x1.0p-160;
}

#endif /* LPG_DETMATH_H */
