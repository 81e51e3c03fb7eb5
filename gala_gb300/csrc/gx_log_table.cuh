// gx_log_table.cuh -- generated by gen_log_table.py; do not edit.
// Constants of the table-driven FP64 logarithm (log_f in gx_fast64.cuh):
// for c_j = 1 + j/64, j = 0..64: {1 / c_j, ln(c_j) high part, ln(c_j) low part}.
#pragma once

namespace gx {
namespace fast {

static __device__ const double LOG_TAB[65][3] = {
    {0x1.0000000000000p+0, 0x0.0p+0, 0x0.0p+0},  // j = 0
    {0x1.f81f81f81f820p-1, 0x1.fc0a8b0fc03e4p-7, -0x1.83092c59642a1p-62},  // j = 1
    {0x1.f07c1f07c1f08p-1, 0x1.f829b0e783300p-6, 0x1.33e3f04f1ef23p-60},  // j = 2
    {0x1.e9131abf0b767p-1, 0x1.77458f632dcfcp-5, 0x1.18d3ca87b9296p-59},  // j = 3
    {0x1.e1e1e1e1e1e1ep-1, 0x1.f0a30c01162a6p-5, 0x1.85f325c5bbacdp-59},  // j = 4
    {0x1.dae6076b981dbp-1, 0x1.341d7961bd1d1p-4, -0x1.b599f227becbbp-58},  // j = 5
    {0x1.d41d41d41d41dp-1, 0x1.6f0d28ae56b4cp-4, -0x1.906d99184b992p-58},  // j = 6
    {0x1.cd85689039b0bp-1, 0x1.a926d3a4ad563p-4, 0x1.942f48aa70ea9p-58},  // j = 7
    {0x1.c71c71c71c71cp-1, 0x1.e27076e2af2e6p-4, -0x1.61578001e0162p-60},  // j = 8
    {0x1.c0e070381c0e0p-1, 0x1.0d77e7cd08e59p-3, 0x1.9a5dc5e9030acp-57},  // j = 9
    {0x1.bacf914c1bad0p-1, 0x1.29552f81ff523p-3, 0x1.301771c407dbfp-57},  // j = 10
    {0x1.b4e81b4e81b4fp-1, 0x1.44d2b6ccb7d1ep-3, 0x1.9f4f6543e1f88p-57},  // j = 11
    {0x1.af286bca1af28p-1, 0x1.5ff3070a793d4p-3, -0x1.bc60efafc6f6ep-58},  // j = 12
    {0x1.a98ef606a63bep-1, 0x1.7ab890210d909p-3, 0x1.be36b2d6a0608p-59},  // j = 13
    {0x1.a41a41a41a41ap-1, 0x1.9525a9cf456b4p-3, 0x1.d904c1d4e2e26p-57},  // j = 14
    {0x1.9ec8e951033d9p-1, 0x1.af3c94e80bff3p-3, -0x1.398cff3641985p-58},  // j = 15
    {0x1.999999999999ap-1, 0x1.c8ff7c79a9a22p-3, -0x1.4f689f8434012p-57},  // j = 16
    {0x1.948b0fcd6e9e0p-1, 0x1.e27076e2af2e6p-3, -0x1.61578001e0162p-59},  // j = 17
    {0x1.8f9c18f9c18fap-1, 0x1.fb9186d5e3e2bp-3, -0x1.caaae64f21acbp-57},  // j = 18
    {0x1.8acb90f6bf3aap-1, 0x1.0a324e27390e3p-2, 0x1.7dcfde8061c03p-56},  // j = 19
    {0x1.8618618618618p-1, 0x1.1675cababa60ep-2, 0x1.ce63eab883717p-61},  // j = 20
    {0x1.8181818181818p-1, 0x1.22941fbcf7966p-2, -0x1.76f5eb09628afp-56},  // j = 21
    {0x1.7d05f417d05f4p-1, 0x1.2e8e2bae11d31p-2, -0x1.8f4cdb95ebdf9p-56},  // j = 22
    {0x1.78a4c8178a4c8p-1, 0x1.3a64c556945eap-2, -0x1.c68651945f97cp-57},  // j = 23
    {0x1.745d1745d1746p-1, 0x1.4618bc21c5ec2p-2, 0x1.f42decdeccf1dp-56},  // j = 24
    {0x1.702e05c0b8170p-1, 0x1.51aad872df82dp-2, 0x1.3927ac19f55e3p-59},  // j = 25
    {0x1.6c16c16c16c17p-1, 0x1.5d1bdbf5809cap-2, 0x1.4236383dc7fe1p-56},  // j = 26
    {0x1.6816816816817p-1, 0x1.686c81e9b14afp-2, -0x1.ddea0f7f58e3dp-57},  // j = 27
    {0x1.642c8590b2164p-1, 0x1.739d7f6bbd007p-2, -0x1.8c76ceb014b04p-56},  // j = 28
    {0x1.6058160581606p-1, 0x1.7eaf83b82afc3p-2, 0x1.92ce979ed2950p-56},  // j = 29
    {0x1.5c9882b931057p-1, 0x1.89a3386c1425bp-2, -0x1.29639dfbbf0fbp-56},  // j = 30
    {0x1.58ed2308158edp-1, 0x1.947941c2116fbp-2, -0x1.16cc8bae0bbe4p-56},  // j = 31
    {0x1.5555555555555p-1, 0x1.9f323ecbf984cp-2, -0x1.a92e513217f5cp-59},  // j = 32
    {0x1.51d07eae2f815p-1, 0x1.a9cec9a9a084ap-2, -0x1.cadec02b436afp-56},  // j = 33
    {0x1.4e5e0a72f0539p-1, 0x1.b44f77bcc8f63p-2, -0x1.cd04495459c78p-56},  // j = 34
    {0x1.4afd6a052bf5bp-1, 0x1.beb4d9da71b7cp-2, -0x1.0f3c590a887cap-59},  // j = 35
    {0x1.47ae147ae147bp-1, 0x1.c8ff7c79a9a22p-2, -0x1.4f689f8434012p-56},  // j = 36
    {0x1.446f86562d9fbp-1, 0x1.d32fe7e00ebd5p-2, 0x1.877b232fafa37p-56},  // j = 37
    {0x1.4141414141414p-1, 0x1.dd46a04c1c4a1p-2, -0x1.0467656d8b892p-56},  // j = 38
    {0x1.3e22cbce4a902p-1, 0x1.e744261d68788p-2, -0x1.c825c90c344b9p-58},  // j = 39
    {0x1.3b13b13b13b14p-1, 0x1.f128f5faf06edp-2, -0x1.328df13bb38c3p-56},  // j = 40
    {0x1.3813813813814p-1, 0x1.faf588f78f31fp-2, -0x1.328260d8abca0p-57},  // j = 41
    {0x1.3521cfb2b78c1p-1, 0x1.02552a5a5d0ffp-1, -0x1.cb1cb51408c00p-56},  // j = 42
    {0x1.323e34a2b10bfp-1, 0x1.0723e5c1cdf40p-1, 0x1.395e58e2445bbp-55},  // j = 43
    {0x1.2f684bda12f68p-1, 0x1.0be72e4252a83p-1, -0x1.259da11330801p-55},  // j = 44
    {0x1.2c9fb4d812ca0p-1, 0x1.109f39e2d4c97p-1, -0x1.0e09b27a4373ap-60},  // j = 45
    {0x1.29e4129e4129ep-1, 0x1.154c3d2f4d5eap-1, -0x1.59c33171a6876p-55},  // j = 46
    {0x1.27350b8812735p-1, 0x1.19ee6b467c96fp-1, -0x1.9d1a11443f10cp-56},  // j = 47
    {0x1.2492492492492p-1, 0x1.1e85f5e7040d0p-1, 0x1.ef62cd2f9f1e3p-56},  // j = 48
    {0x1.21fb78121fb78p-1, 0x1.23130d7bebf43p-1, -0x1.f48725e374d6ep-55},  // j = 49
    {0x1.1f7047dc11f70p-1, 0x1.2795e1289b11bp-1, -0x1.487c0c246978ep-57},  // j = 50
    {0x1.1cf06ada2811dp-1, 0x1.2c0e9ed448e8cp-1, -0x1.1a158f3917586p-55},  // j = 51
    {0x1.1a7b9611a7b96p-1, 0x1.307d7334f10bep-1, 0x1.fb590a1f566dap-57},  // j = 52
    {0x1.1811811811812p-1, 0x1.34e289d9ce1d3p-1, 0x1.6eb92d885ce4fp-57},  // j = 53
    {0x1.15b1e5f75270dp-1, 0x1.393e0d3562a1ap-1, -0x1.58eef67f2483ap-55},  // j = 54
    {0x1.135c81135c811p-1, 0x1.3d9026a7156fbp-1, -0x1.6fef670bd4b62p-55},  // j = 55
    {0x1.1111111111111p-1, 0x1.41d8fe84672aep-1, 0x1.9192f30bd1806p-55},  // j = 56
    {0x1.0ecf56be69c90p-1, 0x1.4618bc21c5ec2p-1, 0x1.f42decdeccf1dp-55},  // j = 57
    {0x1.0c9714fbcda3bp-1, 0x1.4a4f85db03ebbp-1, 0x1.13dfa3d3761b6p-60},  // j = 58
    {0x1.0a6810a6810a7p-1, 0x1.4e7d811b75bb1p-1, -0x1.8d3d9ea6e9ea9p-55},  // j = 59
    {0x1.0842108421084p-1, 0x1.52a2d265bc5abp-1, -0x1.1883750ea4d0ap-57},  // j = 60
    {0x1.0624dd2f1a9fcp-1, 0x1.56bf9d5b3f399p-1, 0x1.0471885cd8ff3p-55},  // j = 61
    {0x1.0410410410410p-1, 0x1.5ad404c359f2dp-1, -0x1.35955683f7196p-59},  // j = 62
    {0x1.0204081020408p-1, 0x1.5ee02a9241675p-1, 0x1.c358257f49082p-55},  // j = 63
    {0x1.0000000000000p-1, 0x1.62e42fefa39efp-1, 0x1.abc9e3b39803fp-56},  // j = 64
};

constexpr double LN2_HI = 0x1.62e42ff000000p-1;  // 32 significant bits
constexpr double LN2_LO = -0x1.718432a1b0e26p-35;

}  // namespace fast
}  // namespace gx

