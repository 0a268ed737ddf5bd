// Drop-in interface: the location / existence enums of the original containers
// (location_enums.h of Batched-ILU0-merged/ILU0_ISAI_bicgstab).  Same names and
// enumerators so that code written against the original links against bilu.
#pragma once

enum class LOCATION { CPU, GPU };
enum class CPU_EXISTENCE { NON_EXISTENT, EXISTENT };
enum class GPU_EXISTENCE { NON_EXISTENT, EXISTENT };
