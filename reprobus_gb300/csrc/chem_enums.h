// chem_enums.h — numbering of the photolysis rates (src/reprobus_l137_20230723.f:754-794)
// and of the thermal rate constants (order of :930-1303), 0-based. Plain C++,
// shared by the device code and host-side checks.
#pragma once

namespace rpb {

// photolysis indices, F:754-794 (0-based)
enum {
    J_o2, J_no2, J_o3_o1d, J_o3_o3p, J_no3_no, J_no3_no2, J_n2o5, J_hno3, J_hno4, J_h2o2,
    J_h2o, J_n2o, J_hocl, J_clono2_cl, J_clono2_clo, J_cl2o2, J_hcl, J_cl2, J_clno2, J_bro,
    J_brono2, J_hobr, J_oclo, J_brcl, J_ch3o2h, J_ch2o_hco, J_ch2o_co, J_cfc11, J_cfc12,
    J_cfc113, J_ccl4, J_ch3ccl3, J_ch3cl, J_hcfc22, J_ch3br, J_h1211, J_h1301, J_co2,
    J_ch2br2, J_hbr, J_no
};

// rate-constant indices, order of F:930-1303 (matches REPROBUS_DIAG_RATE)
enum {
    K_a1, K_a1et, K_a2, K_a5, K_a6, K_a6b, K_a7, K_a17, K_a19, K_a26, K_a27, K_a30, K_a31, K_a36,
    K_b3, K_b4, K_b6, K_b7, K_b9, K_b12, K_b22, K_b23, K_b24, K_b27, K_b28, K_b32, K_b38, K_b39,
    K_c1a, K_c1b, K_c1c, K_c2, K_c3, K_c4, K_c5, K_c7, K_c8, K_c9, K_c10, K_c12, K_c14, K_c15,
    K_c17a, K_c17b, K_c18, K_c19,
    K_d2, K_d3, K_d4, K_d5, K_d6, K_d7, K_d8, K_d9, K_d10, K_d11, K_d31, K_d32, K_d33, K_d34,
    K_d35, K_d36, K_d37, K_d60, K_d61, K_d62, K_d90, K_d91, K_d92, K_d93, K_d94, K_d95, K_d96,
    K_d97,
    K_e2, K_e3, K_e4, K_e5a, K_e5b, K_e5c, K_e6, K_e7, K_e8, K_e9, K_e10, K_e11, K_e13, K_e15,
    K_e16, K_e50, K_e51, K_e52, K_e53, K_e54,
    K_hk1, K_hk2, K_hk3, K_hk4, K_hk5,
    K_COUNT
};
static_assert(K_COUNT == 99, "rate count");

}  // namespace rpb
