// Prints the byte layout of the reference's CSF_cuda object
// (pdflow_cudalib.h:38-154) as a C header, so that the harness in
// refharness.c can fill the object image that the reference kernels read.
// Compiled against the reference header by oracle/ref/Makefile; the header it
// writes holds offsets only.
#include "pdflow_cudalib.h"
#include <cstddef>
#include <cstdio>

#define OFF(f) std::printf("#define CSF_OFF_%s %zu\n", #f, offsetof(CSF_cuda, f));

int main()
{
    std::printf("/* generated by oracle/ref/layout_gen.cu from the reference header */\n");
    std::printf("#define CSF_SIZEOF %zu\n", sizeof(CSF_cuda));
    OFF(rows) OFF(cols) OFF(ctf_levels) OFF(cam_mode) OFF(lambda_i) OFF(lambda_d) OFF(mu) OFF(fovh) OFF(fovv)
    OFF(local_level) OFF(level_image) OFF(rows_i) OFF(cols_i) OFF(g_mask_dev) OFF(colour_wf_dev) OFF(depth_wf_dev)
    OFF(depth_old_dev) OFF(xx_old_dev) OFF(yy_old_dev) OFF(depth_dev) OFF(xx_dev) OFF(yy_dev)
    OFF(colour_old_dev) OFF(colour_dev) OFF(dx_dev) OFF(dy_dev) OFF(dz_dev)
    OFF(dcu_aux_dev) OFF(dcv_aux_dev) OFF(ddu_aux_dev) OFF(ddv_aux_dev)
    OFF(dct_dev) OFF(dcu_dev) OFF(dcv_dev) OFF(ddt_dev) OFF(ddu_dev) OFF(ddv_dev)
    OFF(gradu1_dev) OFF(gradu2_dev) OFF(gradv1_dev) OFF(gradv2_dev) OFF(gradw1_dev) OFF(gradw2_dev)
    OFF(divpu_dev) OFF(divpv_dev) OFF(divpw_dev)
    OFF(sigma_pd_dev) OFF(sigma_puvx_dev) OFF(sigma_puvy_dev) OFF(sigma_pwx_dev) OFF(sigma_pwy_dev)
    OFF(tau_u_dev) OFF(tau_v_dev) OFF(tau_w_dev)
    OFF(mu_uv_dev) OFF(ri_dev) OFF(rj_dev) OFF(ri_2_dev) OFF(rj_2_dev)
    OFF(du_acc_dev) OFF(dv_acc_dev) OFF(dw_acc_dev) OFF(du_prev_dev) OFF(dv_prev_dev)
    OFF(du_upsamp_dev) OFF(dv_upsamp_dev) OFF(dw_upsamp_dev) OFF(pd_upsamp_dev)
    OFF(puu_upsamp_dev) OFF(puv_upsamp_dev) OFF(pvu_upsamp_dev) OFF(pvv_upsamp_dev)
    OFF(pwu_upsamp_dev) OFF(pwv_upsamp_dev)
    OFF(du_l_dev) OFF(dv_l_dev) OFF(dw_l_dev) OFF(pd_l_dev) OFF(puu_l_dev) OFF(puv_l_dev)
    OFF(pvu_l_dev) OFF(pvv_l_dev) OFF(pwu_l_dev) OFF(pwv_l_dev)
    OFF(du_new_dev) OFF(dv_new_dev) OFF(dw_new_dev) OFF(pd_dev) OFF(puu_dev) OFF(puv_dev)
    OFF(pvu_dev) OFF(pvv_dev) OFF(pwu_dev) OFF(pwv_dev)
    return 0;
}
