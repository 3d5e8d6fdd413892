// Convolutional PML of the open boundaries (fields/absorber/pml): device view and the
// host-side coefficient tables.  Not part of the C-ABI.
#pragma once

#include "picgb_internal.hpp"

#include <cmath>
#include <vector>

namespace picgb
{
    // components of the convolution fields psiE and psiB, each nx*ny*nz floats:
    // psi.ab belongs to field component a and the derivative along b (Pml.kernel naming)
    enum PsiComponent
    {
        kPsiXY = 0,
        kPsiXZ = 1,
        kPsiYX = 2,
        kPsiYZ = 3,
        kPsiZX = 4,
        kPsiZY = 5
    };

    struct PmlDev
    {
        float* psiE; // 6 * ncell
        float* psiB; // 6 * ncell
        float const* tab; // [2 fields][3 axes][b, c, kappa][nmax]; E at cell i, B at cell i + 1/2
        int nmax; // largest cell count over the axes
    };

    // Parameters of one axis (param/fieldAbsorber.param).
    struct PmlAxis
    {
        bool open = false;
        int cells = 0; // cells along the axis
        int neg = 0, pos = 0; // PML thickness at the negative and positive face
        double sigmaMax = 0.0, kappaMax = 1.0, alphaMax = 0.0, order = 4.0, alphaOrder = 1.0;
    };

    // b, c, kappa at position x (in cells) along one axis, in double (Pml.kernel:130-267):
    // relative depth d into the layer, sigma = sigmaMax d^m, kappa = 1 + (kappaMax - 1) d^m,
    // alpha = alphaMax (1 - d)^ma, b = exp(-(sigma / kappa + alpha) dt),
    // c = sigma (b - 1) / (kappa (sigma + alpha kappa)) (0 where that denominator is 0).
    inline void pmlCoefficients(PmlAxis const& a, double x, double dt, double& b, double& c, double& k)
    {
        double depth = 0.0;
        if(a.open)
        {
            double const rightStart = double(a.cells - a.pos);
            if(x < double(a.neg))
                depth = (double(a.neg) - x) / double(a.neg);
            else if(x > rightStart && a.pos > 0)
                depth = (x - rightStart) / double(a.pos);
        }
        double sigma = 0.0, alpha = 0.0;
        k = 1.0;
        if(depth != 0.0)
        {
            double const grade = std::pow(depth, a.order);
            sigma = a.sigmaMax * grade;
            k = 1.0 + (a.kappaMax - 1.0) * grade;
            alpha = a.alphaMax * std::pow(1.0 - depth, a.alphaOrder);
        }
        b = std::exp(-(sigma / k + alpha) * dt);
        double const den = k * (sigma + alpha * k);
        c = den != 0.0 ? sigma * (b - 1.0) / den : 0.0;
    }

    // The tables of PmlDev::tab, rounded to float.
    inline std::vector<float> pmlTables(PmlAxis const ax[3], double dt, int nmax)
    {
        std::vector<float> t(size_t(2 * 3 * 3) * nmax, 0.0f);
        for(int f = 0; f < 2; ++f)
            for(int a = 0; a < 3; ++a)
                for(int i = 0; i < nmax; ++i)
                {
                    double b = 1.0, c = 0.0, k = 1.0;
                    if(i < ax[a].cells)
                        pmlCoefficients(ax[a], double(i) + (f ? 0.5 : 0.0), dt, b, c, k);
                    float* row = t.data() + size_t((f * 3 + a) * 3) * nmax;
                    row[i] = float(b);
                    row[nmax + i] = float(c);
                    row[2 * nmax + i] = float(k);
                }
        return t;
    }

    // Damping factor per axis and cell of the exponential absorber (Exponential.kernel:50-90): a
    // cell f = 1 .. thickness - 1 cells deep into a face's layer (counted from the layer's inner
    // edge) is multiplied by exp(-strength f); 1 elsewhere.  Rounded to float from double.
    inline std::vector<float> expDampTable(int const cells[3], int const thick[3][2], float const strength[3][2], int open, int nmax)
    {
        std::vector<float> t(size_t(3) * nmax, 1.0f);
        for(int a = 0; a < 3; ++a)
        {
            if(!(open & (1 << a)))
                continue;
            for(int i = 0; i < cells[a]; ++i)
            {
                double d = 1.0;
                int const fNeg = thick[a][0] - 1 - i;
                if(fNeg > 0)
                    d *= std::exp(-double(strength[a][0]) * double(fNeg));
                int const fPos = i - cells[a] + thick[a][1];
                if(fPos > 0)
                    d *= std::exp(-double(strength[a][1]) * double(fPos));
                t[size_t(a) * nmax + i] = float(d);
            }
        }
        return t;
    }

    // F *= damp_x(x), then *= damp_y(y), then *= damp_z(z), each factor != 1 one rounding step
    cudaError_t launchAbsorbExponential(float* F, GridParams const& g, float const* damp, int nmax, cudaStream_t stream);

    cudaError_t launchYeeBHalfOpen(float const* E, float* B, GridParams const& g, PmlDev const& p, bool updatePsi, cudaStream_t stream);
    cudaError_t launchYeeEOpen(
        float const* B,
        float* E,
        float const* J,
        float coeff,
        GridParams const& g,
        PmlDev const& p,
        cudaStream_t stream);
} // namespace picgb
