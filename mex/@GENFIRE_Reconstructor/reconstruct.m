function obj = reconstruct(obj)
% Replaces @GENFIRE_Reconstructor/reconstruct.m: the iteration on the GPU through
% genfire_mex.c and libgenfire.so (genfire_reconstruct).
if obj.calculate_Rfree == 1
    % the withheld points are drawn here, with MATLAB's own rng and randperm
    % (reconstruct.m:46-67); the library finds the candidates and monitors them
    cand = genfire_mex('rfree_candidates', obj);
    R_freeInd = cell(1, numel(cand));
    for s = 1:numel(cand)
        if ~isempty(obj.RandomSeed), rng(obj.RandomSeed); end
        c = cand{s}(randperm(numel(cand{s})));
        cut = floor(numel(c) .* obj.percentValuesForRfree);
        if cut == 0, cut = 1; end
        R_freeInd{s} = c(1:cut);
        obj.measuredK_mask(R_freeInd{s}) = false;
    end
    [obj.reconstruction, obj.errK, obj.errR, obj.Rarr_record, obj.Rarr2_record, rf] = ...
        genfire_mex('reconstruct_rfree', obj, R_freeInd);
    obj.Rfree_complex = single(rf);
else
    [obj.reconstruction, obj.errK, obj.errR, obj.Rarr_record, obj.Rarr2_record] = genfire_mex('reconstruct', obj);
end
end
