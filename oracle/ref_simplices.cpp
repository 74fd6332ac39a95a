// Test-infrastructure probe: prints the reference's simplicial decomposition of the unit hypercube
// (MishaK::HyperCubeSimplices<Dim>, Misha/HyperCubeSimplices.h:51-185, as
// MarchingSimplices::RegularSubGridTriangulation orients it, Misha/MarchingSimplices.h:623-660) so
// that the oracle's restatement of the reference's zero-set extraction uses the same simplices.
// Output: one line per simplex, Dim+1 vertices, each vertex its Dim 0/1 coordinates.
#include <cstdio>
#include "Misha/Geometry.h"
#include "Misha/MarchingSimplices.h"

using namespace MishaK;

template <unsigned int Dim>
static void Dump()
{
    HyperCubeSimplices<Dim> hcs;
    printf("dim %u simplices %u\n", Dim, HyperCubeSimplices<Dim>::SimplexNum);
    for (unsigned int i = 0; i < HyperCubeSimplices<Dim>::SimplexNum; i++)
    {
        Simplex<unsigned int, Dim, Dim> s = hcs.simplex(i);
        SquareMatrix<double, Dim> M;
        for (unsigned int j = 0; j < Dim; j++)
            for (unsigned int k = 0; k < Dim; k++) M(j, k) = (double)s[j + 1][k] - (double)s[0][k];
        if (M.determinant() < 0) std::swap(s[0], s[1]);
        for (unsigned int j = 0; j <= Dim; j++)
            for (unsigned int d = 0; d < Dim; d++) printf("%u%s", s[j][d], (j == Dim && d == Dim - 1) ? "\n" : " ");
    }
}

int main()
{
    Dump<3>();
    Dump<4>();
    return 0;
}
