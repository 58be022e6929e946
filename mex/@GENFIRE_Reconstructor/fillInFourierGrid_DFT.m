function obj = fillInFourierGrid_DFT(obj)
% Replaces @GENFIRE_Reconstructor/fillInFourierGrid_DFT.m: DFT gridding on the GPU
% through genfire_mex.c and libgenfire.so (genfire_grid_dft).
[obj.measuredK, obj.recIFFT] = genfire_mex('grid_dft', obj);
end
