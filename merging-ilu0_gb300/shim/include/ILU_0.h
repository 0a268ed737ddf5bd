// Drop-in interface: ILU_0.h of the original code (ILU(0) of a paged batch
// into separate L / U pages; in-place approach-1 factorisation).
#pragma once

class PagedCSRMatrices;

void ILU_0_Factorization_Gpu(const PagedCSRMatrices& A_pages, PagedCSRMatrices& L_pages, PagedCSRMatrices& U_pages,
                             const int approach_num);
void ComputeILU0Approach1(PagedCSRMatrices& Factored_Pages, const int* const diag_ptrs);
