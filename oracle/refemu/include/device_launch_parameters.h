#pragma once
// CPU emulation: built-in variables are declared in cuda_runtime.h
