// Localization regions of one task on the host (LocalizationRegions,
// src/LocalizationRegions.cc): moving the centres toward the orbitals'
// centres and setting the radii from their spreads, with the reference's
// arithmetic, so that the mask sets can be rebuilt for the new regions
// (mgx_masks_update).
#include <cmath>

#include "mgx_internal.cuh"

extern "C" {

/* LocalizationRegions::moveTo (src/LocalizationRegions.cc:405-450) with the
 * minimum-image vector of Vector3D::vminimage (src/tools/Vector3D.cc:32-63,
 * periodic): each centre moves toward its target by the minimum-image
 * difference, shortened to 1 bohr when longer; *max_displ receives the
 * longest difference before shortening. */
int mgx_regions_move_to(int nfunc, double* centers, const double* targets, const double cell[3],
    float* max_displ)
{
    if (nfunc < 0 || (nfunc > 0 && (!centers || !targets)) || !cell || !max_displ)
        return mgx::fail(MGX_BAD_ARG, "regions: NULL argument");
    for (int i = 0; i < 3; i++)
        if (!(cell[i] > 0.)) return mgx::fail(MGX_BAD_ARG, "regions: cell");
    float mx = 0.f;
    for (int f = 0; f < nfunc; f++)
    {
        double d[3];
        for (int i = 0; i < 3; i++)
        {
            double r         = std::fmod(targets[3 * f + i] - centers[3 * f + i], cell[i]);
            const double ax2 = 0.5 * cell[i];
            if (r > ax2)
                r -= cell[i];
            else if (r < -ax2)
                r += cell[i];
            d[i] = r;
        }
        const float nrm = (float)std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
        if (nrm > mx) mx = nrm;
        if (nrm > 1.)
            for (int i = 0; i < 3; i++)
                d[i] /= nrm;
        for (int i = 0; i < 3; i++)
            centers[3 * f + i] += d[i];
    }
    *max_displ = mx;
    return MGX_OK;
}

/* LocalizationRegions::updateRadii(sc, ratio) (:354-366): radius_j = ratio
 * spread_j, stored as float; *mean_radius receives getMeanRadius (:332-352),
 * the cube root of the mean cube of the radii. */
int mgx_regions_update_radii(int nfunc, const double* spreads, float ratio, float* radii,
    float* mean_radius)
{
    if (nfunc <= 0 || !spreads || !radii || !mean_radius)
        return mgx::fail(MGX_BAD_ARG, "regions: NULL argument");
    float rcube = 0.f;
    for (int f = 0; f < nfunc; f++)
    {
        radii[f]          = (float)(ratio * spreads[f]);
        const float alpha = radii[f];
        rcube += (alpha * alpha * alpha);
    }
    *mean_radius = std::cbrt(rcube / (float)nfunc);
    return MGX_OK;
}

} // extern "C"
