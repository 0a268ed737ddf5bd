// Drop-in interface: parILU_0.h of the original code.
#pragma once

class PagedCSRMatrices;

void ParILU_0_Factorization_Gpu(const PagedCSRMatrices& A_pages, PagedCSRMatrices& L_pages,
                                PagedCSRMatrices& U_pages, const int num_iterations);
